/* CPU oracle for the MSCEER lower-star discrete gradient (.grad) path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference algorithm
 * that the tests, bench.py's CPU baseline legs and __graft_entry__.smoke() use
 * as the checker for the CUDA path.  The product never links or calls it.
 *
 * It restates, step for step (file:line in the MSCEER reference):
 *   - the cell complex index algebra of TopologicalRegularGrid3D/2D
 *       (gi_topological_regular_grid.h:113-342, 1182-1341; 2D :1952-2241)
 *   - highest/lowest vertex of a cell under the (value, then vertex index) order
 *       RegularGridMaxMinVertexLabeling3D::ComputeOutput + Before
 *       (gi_max_vertex_labeling.h:758-760, 771-889) and IsGreater
 *       (gi_regular_grid_trilinear_function.h:309-314)
 *   - the relaxed Robins lower-star pairing of every vertex with the star split by
 *       cell boundaryValue: MyRobinsNoalloc::ComputeLowerStar/HomotopyExpand
 *       (gi_modified_robins.h:1281-1343, 999-1199).  For interior vertices every
 *       star cell has boundaryValue 0, so this is the same computation as
 *       SlidingWindowRobinsNoalloc::ComputeLowerStar/HomotopyExpand
 *       (gi_fast_robins_noalloc.h:353-428, 147-321) that steepest_lstar runs there.
 *   - setAscendingManifoldDimensions + rec_man_trace_up_marking
 *       (gi_topological_gradient_using_algorithms.h:395-478)
 *   - the boundary flag written by DiscreteGradientLabeling::outputToFile
 *       (gi_discrete_gradient_labeling.h:200-226)
 * Byte layout: GradBitfield (gi_discrete_gradient_labeling.h:11-19), LSB first:
 * assigned:1 flag:1 pair:3 ldir:3.
 *
 * Parity of this restatement is pinned against the reference compiled from its
 * own sources (oracle/ref_harness.cpp) and the committed golden .grad files.
 * Inputs containing NaN are outside the contract (the reference's own result then
 * depends on its reduction order).
 */
#include "msc_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
	int nd;              /* 2 or 3 */
	int64_t v[3];        /* vertices per axis */
	int64_t d[3];        /* cells per axis = 2v-1 */
	int64_t cs[3];       /* cell-id stride per axis */
	int64_t vs[3];       /* vertex-index stride per axis */
	int64_t ncells;
} mesh_t;

static int mesh_init(mesh_t* m, int nd, int64_t X, int64_t Y, int64_t Z) {
	if (X < 1 || Y < 1 || Z < 1) return -1;
	m->nd = nd;
	m->v[0] = X; m->v[1] = Y; m->v[2] = (nd == 3) ? Z : 1;
	for (int a = 0; a < 3; a++) m->d[a] = 2 * m->v[a] - 1;
	m->cs[0] = 1; m->cs[1] = m->d[0]; m->cs[2] = m->d[0] * m->d[1];
	m->vs[0] = 1; m->vs[1] = m->v[0]; m->vs[2] = m->v[0] * m->v[1];
	m->ncells = m->d[0] * m->d[1] * m->d[2];
	return 0;
}

static inline void cell_coords(const mesh_t* m, int64_t id, int64_t c[3]) {
	/* cellid2Coords, gi_topological_regular_grid.h:1268-1272 */
	c[0] = id % m->d[0];
	c[1] = (id / m->d[0]) % m->d[1];
	c[2] = id / (m->d[0] * m->d[1]);
}

static inline int64_t cell_id(const mesh_t* m, const int64_t c[3]) {
	return c[0] + c[1] * m->cs[1] + c[2] * m->cs[2];
}

/* VertexNumberFromCellID (gi_topological_regular_grid.h:1337-1341) */
static inline int64_t vertex_number(const mesh_t* m, int64_t id) {
	int64_t c[3];
	cell_coords(m, id, c);
	return (c[0] >> 1) * m->vs[0] + (c[1] >> 1) * m->vs[1] + (c[2] >> 1) * m->vs[2];
}

static inline int cell_dim(const mesh_t* m, const int64_t c[3]) {
	int s = 0;
	for (int a = 0; a < m->nd; a++) s += (int)(c[a] & 1);
	return s;
}

static inline int boundary_value(const mesh_t* m, const int64_t c[3]) {
	/* boundaryValue for a non-periodic mesh, gi_topological_regular_grid.h:1291-1297 */
	int s = 0;
	for (int a = 0; a < m->nd; a++) s += (c[a] == 0 || c[a] == m->d[a] - 1);
	return s;
}

/* a comes before b in the (value, then index) vertex order: IsGreater(b, a). */
static inline int before(const float* f, int64_t a, int64_t b) {
	if (f[b] > f[a]) return 1;
	if (f[a] > f[b]) return 0;
	return b > a;
}

/* Highest (want_max) or lowest vertex index of the cell at coords c. */
static int64_t extreme_vertex(const mesh_t* m, const float* f, const int64_t c[3], int want_max) {
	int odd[3], nodd = 0;
	for (int a = 0; a < m->nd; a++) if (c[a] & 1) odd[nodd++] = a;
	int64_t best = -1;
	for (int s = 0; s < (1 << nodd); s++) {
		int64_t vc[3] = { c[0], c[1], c[2] };
		for (int t = 0; t < nodd; t++) vc[odd[t]] += ((s >> t) & 1) ? 1 : -1;
		int64_t vi = (vc[0] >> 1) * m->vs[0] + (vc[1] >> 1) * m->vs[1] + (vc[2] >> 1) * m->vs[2];
		if (best < 0) { best = vi; continue; }
		if (want_max ? before(f, best, vi) : before(f, vi, best)) best = vi;
	}
	return best;
}

/* Facets in TopologicalRegularGrid3D::FacetsIterator order: +x,-x,+y,-y,+z,-z over odd axes. */
static int facets(const mesh_t* m, int64_t id, const int64_t c[3], int64_t out[6]) {
	int n = 0;
	for (int a = 0; a < m->nd; a++) {
		if (c[a] & 1) { out[n++] = id + m->cs[a]; out[n++] = id - m->cs[a]; }
	}
	return n;
}

/* Cofacets in CofacetsIterator order: +x,-x,+y,-y,+z,-z over even axes, in bounds only
 * (gi_topological_regular_grid.h:312-340, 555-591). */
static int cofacets(const mesh_t* m, int64_t id, const int64_t c[3], int64_t out[6]) {
	int n = 0;
	for (int a = 0; a < m->nd; a++) {
		if (!(c[a] & 1)) {
			if (c[a] != m->d[a] - 1) out[n++] = id + m->cs[a];
			if (c[a] != 0) out[n++] = id - m->cs[a];
		}
	}
	return n;
}

/* Compress6NeighborOffsetToByte (gi_topological_regular_grid.h:1182-1192); the 2D
 * mesh's m_offset_2_direction_map gives the same codes 0..3 for +x,-x,+y,-y. */
static inline uint8_t pair_code(const mesh_t* m, int64_t base, int64_t other) {
	int64_t diff = other - base;
	if (m->nd == 2) {
		/* m_offset_2_direction_map (gi_topological_regular_grid.h:2232-2241) inserts the
		 * +x,-x,+y,-y offsets and their wraparound offsets in that order; a later key
		 * overwrites an equal earlier one (only when X == 1, where +x and +y coincide). */
		const int64_t adj[4] = { 1, -1, m->d[0], -m->d[0] };
		const int64_t wrap[4] = { -(m->d[0] - 1), m->d[0] - 1, -(m->d[1] - 1) * m->d[0], (m->d[1] - 1) * m->d[0] };
		for (int i = 3; i >= 0; i--) if (adj[i] == diff || wrap[i] == diff) return (uint8_t)i;
		return 0;  /* operator[] on a missing key default-inserts 0 */
	}
	int neg = diff < 0;
	int64_t ad = neg ? -diff : diff;
	if (ad == m->cs[0]) return (uint8_t)(0 + neg);
	if (ad == m->cs[1]) return (uint8_t)(2 + neg);
	if (m->nd == 3 && ad == m->cs[2]) return (uint8_t)(4 + neg);
	return 7;
}

static inline int64_t decode_pair(const mesh_t* m, int64_t base, uint8_t code) {
	/* UncompressByteTo6NeighborOffset: base + m_adjacency_offsets[code] */
	int64_t off = m->cs[code >> 1];
	return (code & 1) ? base - off : base + off;
}

#define GB_ASSIGNED 0x01u
#define GB_FLAG     0x02u
#define GB_PAIR_SH  2
#define GB_PAIR_MSK (0x7u << GB_PAIR_SH)
#define GB_LDIR_SH  5
#define GB_LDIR_MSK (0x7u << GB_LDIR_SH)

/* One boundary class of one vertex's lower star: the cp/list structures of
 * MyRobinsNoalloc::HomotopyExpand (gi_modified_robins.h:999-1199). */
typedef struct {
	int n;
	int64_t id[27];
	int64_t c[27][3];
	int dim[27];
	int num_missing[27];
	int pair[27];       /* list index of the partner, itself if critical */
	int paired[27];
	int64_t lowv[27];   /* lowest vertex, computed lazily */
} lstar_t;

static int find_in(const lstar_t* L, int64_t id) {
	for (int i = 0; i < L->n; i++) if (L->id[i] == id) return i;
	return -1;
}

static void decrement_cofacets(const mesh_t* m, lstar_t* L, int i) {
	int64_t cf[6];
	int ncf = cofacets(m, L->id[i], L->c[i], cf);
	for (int t = 0; t < ncf; t++) {
		int j = find_in(L, cf[t]);
		if (j >= 0) L->num_missing[j]--;
	}
}

static int64_t lowest_vertex(const mesh_t* m, const float* f, lstar_t* L, int i) {
	if (L->lowv[i] < 0) L->lowv[i] = extreme_vertex(m, f, L->c[i], 0);
	return L->lowv[i];
}

/* PickLowestCandidate (gi_modified_robins.h:777-794): the first candidate wins ties. */
static int pick_lowest(const mesh_t* m, const float* f, lstar_t* L, const int* cand, int nc) {
	if (nc == 1) return cand[0];
	int cur = cand[0];
	int64_t lv = lowest_vertex(m, f, L, cur);
	for (int i = 1; i < nc; i++) {
		int64_t olv = lowest_vertex(m, f, L, cand[i]);
		if (before(f, olv, lv)) { lv = olv; cur = cand[i]; }
	}
	return cur;
}

static void homotopy_expand(const mesh_t* m, const float* f, int64_t vcell, lstar_t* L) {
	int bydim[4][27], nd_[4] = { 0, 0, 0, 0 };
	for (int i = 0; i < L->n; i++) {
		L->num_missing[i] = 0; L->pair[i] = -1; L->paired[i] = 0; L->lowv[i] = -1;
	}
	for (int i = 0; i < L->n; i++) {
		bydim[L->dim[i]][nd_[L->dim[i]]++] = i;
		int64_t fc[6];
		int nf = facets(m, L->id[i], L->c[i], fc);
		for (int t = 0; t < nf; t++) if (find_in(L, fc[t]) >= 0) L->num_missing[i]++;
	}
	/* the vertex pairs with the edge to its lowest neighbour, or is critical */
	if (nd_[0] > 0) {
		int vl = bydim[0][0];
		if (nd_[1] == 0) {
			L->pair[vl] = vl; L->paired[vl] = 1;
			decrement_cofacets(m, L, vl);
		} else {
			int el = bydim[1][0];
			int64_t fc[6];
			facets(m, L->id[el], L->c[el], fc);
			int64_t cur_vn = vertex_number(m, (fc[0] == vcell) ? fc[1] : fc[0]);
			for (int k = 1; k < nd_[1]; k++) {
				int e = bydim[1][k];
				facets(m, L->id[e], L->c[e], fc);
				int64_t r_vn = vertex_number(m, (fc[0] == vcell) ? fc[1] : fc[0]);
				/* is_steeper (gi_modified_robins.h:745-755) keeps the current edge when its
				 * vertex comes first, otherwise takes the other one */
				int64_t steeper = before(f, cur_vn, r_vn) ? cur_vn : r_vn;
				if (steeper != cur_vn) { el = e; cur_vn = steeper; }
			}
			L->pair[vl] = el; L->paired[vl] = 1;
			L->pair[el] = vl; L->paired[el] = 1;
			decrement_cofacets(m, L, vl);
			decrement_cofacets(m, L, el);
		}
	}
	for (int d = 0; d < 4; d++) {
		int num_processed = 0, total = 0;
		for (int j = 0; j < nd_[d]; j++) if (!L->paired[bydim[d][j]]) total++;
		while (num_processed < total) {
			int start = num_processed;
			for (int j = 0; j < nd_[d]; j++) {
				int ic = bydim[d][j];
				if (L->paired[ic]) continue;
				int cand[6], nc = 0;
				int64_t cf[6];
				int ncf = cofacets(m, L->id[ic], L->c[ic], cf);
				for (int t = 0; t < ncf; t++) {
					int li = find_in(L, cf[t]);
					if (li < 0) continue;
					if (L->num_missing[li] == 1) cand[nc++] = li;
				}
				if (nc > 0) {
					int cfl = pick_lowest(m, f, L, cand, nc);
					L->pair[ic] = cfl; L->paired[ic] = 1;
					L->pair[cfl] = ic; L->paired[cfl] = 1;
					decrement_cofacets(m, L, ic);
					decrement_cofacets(m, L, cfl);
					num_processed++;
					break;
				}
			}
			if (start == num_processed) {
				int cand[27], nc = 0;
				for (int j = 0; j < nd_[d]; j++) {
					int ic = bydim[d][j];
					if (!L->paired[ic]) cand[nc++] = ic;
				}
				int cl = pick_lowest(m, f, L, cand, nc);
				L->pair[cl] = cl; L->paired[cl] = 1;
				decrement_cofacets(m, L, cl);
				num_processed++;
			}
		}
	}
}

static void write_pairs(const mesh_t* m, const lstar_t* L, uint8_t* g) {
	for (int j = 0; j < L->n; j++) {
		int64_t id = L->id[j];
		int p = L->pair[j];
		if (p == j) {
			g[id] = (uint8_t)((g[id] & ~GB_PAIR_MSK) | (7u << GB_PAIR_SH) | GB_ASSIGNED);
		} else {
			int64_t pid = L->id[p];
			g[id] = (uint8_t)((g[id] & ~GB_PAIR_MSK) | ((unsigned)pair_code(m, id, pid) << GB_PAIR_SH) | GB_ASSIGNED);
			g[pid] = (uint8_t)((g[pid] & ~GB_PAIR_MSK) | ((unsigned)pair_code(m, pid, id) << GB_PAIR_SH) | GB_ASSIGNED);
		}
	}
}

/* ComputeLowerStar for one vertex (gi_modified_robins.h:1281-1343): the star split by
 * class restriction_label * maxDim + boundaryValue (maxDim = 3, gi_topological_regular_grid.h:
 * 1262-1264; the label 0 everywhere without a restriction map), the classes expanded in
 * increasing order. */
#define N_CLASSES 24
static void compute_lower_star_r(const mesh_t* m, const float* f, int64_t vx, int64_t vy, int64_t vz, uint8_t* g,
                                 const uint8_t* restrict_lab) {
	int64_t vc[3] = { 2 * vx, 2 * vy, 2 * vz };
	int64_t vcell = cell_id(m, vc);
	int64_t vid = vx * m->vs[0] + vy * m->vs[1] + vz * m->vs[2];
	lstar_t cls[N_CLASSES];
	for (int s = 0; s < N_CLASSES; s++) cls[s].n = 0;
	int npos = (m->nd == 3) ? 27 : 9;
	for (int p = 0; p < npos; p++) {
		/* AdjacentCellsIterator order: x fastest over offsets -1..1 */
		int64_t c[3] = { vc[0] + (p % 3) - 1, vc[1] + (p / 3) % 3 - 1, vc[2] + ((m->nd == 3) ? (p / 9) - 1 : 0) };
		int ok = 1;
		for (int a = 0; a < m->nd; a++) if (c[a] < 0 || c[a] >= m->d[a]) ok = 0;
		if (!ok) continue;
		if (extreme_vertex(m, f, c, 1) != vid) continue;   /* not in the lower star */
		int key = boundary_value(m, c) + (restrict_lab ? 3 * (int)restrict_lab[cell_id(m, c)] : 0);
		if (key > N_CLASSES - 1) key = N_CLASSES - 1;
		lstar_t* L = &cls[key];
		L->id[L->n] = cell_id(m, c);
		L->c[L->n][0] = c[0]; L->c[L->n][1] = c[1]; L->c[L->n][2] = c[2];
		L->dim[L->n] = cell_dim(m, c);
		L->n++;
	}
	for (int s = 0; s < N_CLASSES; s++) {
		if (cls[s].n == 0) continue;
		homotopy_expand(m, f, vcell, &cls[s]);
		write_pairs(m, &cls[s], g);
	}
}

static void compute_lower_star(const mesh_t* m, const float* f, int64_t vx, int64_t vy, int64_t vz, uint8_t* g) {
	compute_lower_star_r(m, f, vx, vy, vz, g, NULL);
}

static int lstar_pairs(const mesh_t* m, const float* f, uint8_t* g, int nthreads) {
	memset(g, 0, (size_t)m->ncells);   /* ClearAllGradient */
	int64_t nv = m->v[0] * m->v[1] * m->v[2];
#ifdef _OPENMP
	if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nthreads)
#else
	(void)nthreads;
#endif
	for (int64_t vi = 0; vi < nv; vi++) {
		int64_t x = vi % m->v[0];
		int64_t y = (vi / m->v[0]) % m->v[1];
		int64_t z = vi / (m->v[0] * m->v[1]);
		compute_lower_star(m, f, x, y, z, g);
	}
	return 0;
}

/* rec_man_trace_up_marking (gi_topological_gradient_using_algorithms.h:395-425). */
static void trace_up(const mesh_t* m, uint8_t* g, int64_t root, unsigned value, int64_t* q) {
	int64_t head = 0, tail = 0;
	q[tail++] = root;
	while (head < tail) {
		int64_t cur = q[head++];
		if (((g[cur] & GB_LDIR_MSK) >> GB_LDIR_SH) == value) continue;
		g[cur] = (uint8_t)((g[cur] & ~GB_LDIR_MSK) | (value << GB_LDIR_SH));
		int64_t c[3], cf[6];
		cell_coords(m, cur, c);
		int ncf = cofacets(m, cur, c, cf);
		for (int t = 0; t < ncf; t++) {
			int64_t tid = cf[t];
			uint8_t b = g[tid];
			unsigned code = (b & GB_PAIR_MSK) >> GB_PAIR_SH;
			if (code == 7 || !(b & GB_ASSIGNED)) continue;
			int64_t tp = decode_pair(m, tid, (uint8_t)code);
			if (tp == cur) continue;
			if (((b & GB_LDIR_MSK) >> GB_LDIR_SH) == value) continue;
			g[tid] = (uint8_t)((b & ~GB_LDIR_MSK) | (value << GB_LDIR_SH));
			q[tail++] = tp;
		}
	}
}

/* setAscendingManifoldDimensions (gi_topological_gradient_using_algorithms.h:430-478). */
static int ldir_mesh(const mesh_t* m, uint8_t* g) {
	int64_t n = m->ncells;
	int64_t* q = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
	if (!q) return -2;
	for (int64_t i = 0; i < n; i++) g[i] = (uint8_t)((g[i] & ~GB_LDIR_MSK) | (3u << GB_LDIR_SH));
	for (int pass = 0; pass < 3; pass++) {
		int want_dim = pass + 1;          /* 1-cells -> 2, 2-cells -> 1, 3-cells -> 0 */
		unsigned value = (unsigned)(2 - pass);
		for (int64_t i = 0; i < n; i++) {
			if (((g[i] & GB_PAIR_MSK) >> GB_PAIR_SH) != 7) continue;
			int64_t c[3];
			cell_coords(m, i, c);
			if (cell_dim(m, c) != want_dim) continue;
			if (want_dim == 3) g[i] = (uint8_t)(g[i] & ~GB_LDIR_MSK);
			else trace_up(m, g, i, value, q);
		}
	}
	free(q);
	return 0;
}

static int flag_mesh(const mesh_t* m, uint8_t* g) {
	for (int64_t i = 0; i < m->ncells; i++) {
		int64_t c[3];
		cell_coords(m, i, c);
		if (boundary_value(m, c)) g[i] |= GB_FLAG; else g[i] &= (uint8_t)~GB_FLAG;
	}
	return 0;
}

int oracle_lstar_pairs_3d(const float* f, int64_t X, int64_t Y, int64_t Z, uint8_t* g, int nt) {
	mesh_t m; if (mesh_init(&m, 3, X, Y, Z)) return -1;
	return lstar_pairs(&m, f, g, nt);
}
int oracle_lstar_pairs_2d(const float* f, int64_t X, int64_t Y, uint8_t* g, int nt) {
	mesh_t m; if (mesh_init(&m, 2, X, Y, 1)) return -1;
	return lstar_pairs(&m, f, g, nt);
}
int oracle_ldir_3d(int64_t X, int64_t Y, int64_t Z, uint8_t* g) {
	mesh_t m; if (mesh_init(&m, 3, X, Y, Z)) return -1;
	return ldir_mesh(&m, g);
}
int oracle_ldir_2d(int64_t X, int64_t Y, uint8_t* g) {
	mesh_t m; if (mesh_init(&m, 2, X, Y, 1)) return -1;
	return ldir_mesh(&m, g);
}
int oracle_flag_3d(int64_t X, int64_t Y, int64_t Z, uint8_t* g) {
	mesh_t m; if (mesh_init(&m, 3, X, Y, Z)) return -1;
	return flag_mesh(&m, g);
}
int oracle_flag_2d(int64_t X, int64_t Y, uint8_t* g) {
	mesh_t m; if (mesh_init(&m, 2, X, Y, 1)) return -1;
	return flag_mesh(&m, g);
}
int oracle_grad_3d(const float* f, int64_t X, int64_t Y, int64_t Z, uint8_t* g, int nt) {
	int rc = oracle_lstar_pairs_3d(f, X, Y, Z, g, nt);
	if (!rc) rc = oracle_ldir_3d(X, Y, Z, g);
	if (!rc) rc = oracle_flag_3d(X, Y, Z, g);
	return rc;
}
int oracle_grad_2d(const float* f, int64_t X, int64_t Y, uint8_t* g, int nt) {
	int rc = oracle_lstar_pairs_2d(f, X, Y, g, nt);
	if (!rc) rc = oracle_ldir_2d(X, Y, g);
	if (!rc) rc = oracle_flag_2d(X, Y, g);
	return rc;
}

/* ---- conforming gradient (ondemandaccurate's accurate 3-manifold .grad) --------- */

/* VertexLabelingToBoundaryLabeling::ComputeMINBoundary (gi_labeling_to_bounary_labeling.h:48-116)
 * with `asc`, then ComputeMAXBoundary (:118-199) with `dsc` (either may be NULL): edges
 * whose two vertices carry different ascending labels (neither -1) get 1, then quads with
 * such an edge, then hexes with such a quad; interior quads whose two hexes' highest
 * vertices differ and carry different descending labels get +2, then interior edges
 * with such a quad, then interior vertices with such an edge.  out: one byte per cell. */
int oracle_boundary_labels_3d(const float* f, int64_t X, int64_t Y, int64_t Z, const int32_t* asc,
                              const int32_t* dsc, uint8_t* out) {
	mesh_t M; if (mesh_init(&M, 3, X, Y, Z)) return -1;
	const mesh_t* m = &M;
	memset(out, 0, (size_t)m->ncells);
	if (asc) {
		for (int dimc = 1; dimc <= 3; dimc++) {
			for (int64_t i = 0; i < m->ncells; i++) {
				int64_t c[3];
				cell_coords(m, i, c);
				if (cell_dim(m, c) != dimc) continue;
				int64_t fc[6];
				int nf = facets(m, i, c, fc);
				if (dimc == 1) {
					int32_t l1 = asc[vertex_number(m, fc[0])], l2 = asc[vertex_number(m, fc[1])];
					if (l1 != -1 && l2 != -1 && l1 != l2) out[i] = 1;
				} else {
					for (int t = 0; t < nf; t++) if (out[fc[t]] == 1) { out[i] = 1; break; }
				}
			}
		}
	}
	if (dsc) {
		for (int dimc = 2; dimc >= 0; dimc--) {
			for (int64_t i = 0; i < m->ncells; i++) {
				int64_t c[3];
				cell_coords(m, i, c);
				if (cell_dim(m, c) != dimc || boundary_value(m, c) != 0) continue;
				int64_t cf[6];
				int ncf = cofacets(m, i, c, cf);
				if (dimc == 2) {
					int64_t c1[3], c2[3];
					cell_coords(m, cf[0], c1);
					cell_coords(m, cf[1], c2);
					int64_t v1 = extreme_vertex(m, f, c1, 1), v2 = extreme_vertex(m, f, c2, 1);
					if (v1 == v2) continue;
					int32_t l1 = dsc[v1], l2 = dsc[v2];
					if (l1 == -1 || l2 == -1) continue;
					if (l1 != l2) out[i] = (uint8_t)(out[i] + 2);
				} else {
					for (int t = 0; t < ncf; t++) if (out[cf[t]] > 1) { out[i] = (uint8_t)(out[i] + 2); break; }
				}
			}
		}
	}
	return 0;
}

/* The re-pairing of ondemandaccurate.cxx:1000-1063: every vertex that is restricted, or
 * whose lower star holds a restricted cell, recomputes its lower star split by
 * restriction label and boundaryValue (MyRobinsNoalloc<...,4,6>::ComputeLowerStar); then
 * RecordGrad (:693-699): setAscendingManifoldDimensions and the boundary flag.  g: the
 * base .grad in, the conforming .grad out. */
int oracle_conform_3d(const float* f, int64_t X, int64_t Y, int64_t Z, const uint8_t* restrict_lab, uint8_t* g,
                      int nthreads) {
	mesh_t M; if (mesh_init(&M, 3, X, Y, Z)) return -1;
	const mesh_t* m = &M;
	int64_t nv = X * Y * Z;
#ifdef _OPENMP
	if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nthreads)
#else
	(void)nthreads;
#endif
	for (int64_t vi = 0; vi < nv; vi++) {
		int64_t x = vi % X, y = (vi / X) % Y, z = vi / (X * Y);
		int64_t vc[3] = { 2 * x, 2 * y, 2 * z };
		int hasdiff = restrict_lab[cell_id(m, vc)] > 0;
		for (int p = 0; p < 27 && !hasdiff; p++) {
			int64_t c[3] = { vc[0] + (p % 3) - 1, vc[1] + (p / 3) % 3 - 1, vc[2] + (p / 9) - 1 };
			int ok = 1;
			for (int a = 0; a < 3; a++) if (c[a] < 0 || c[a] >= m->d[a]) ok = 0;
			if (!ok) continue;
			if (restrict_lab[cell_id(m, c)] > 0 && extreme_vertex(m, f, c, 1) == vi) hasdiff = 1;
		}
		if (hasdiff) compute_lower_star_r(m, f, x, y, z, g, restrict_lab);
	}
	int rc = ldir_mesh(m, g);
	if (!rc) rc = flag_mesh(m, g);
	return rc;
}

/* RegularGridTrilinearFunction::ComputeGradFromImage(1)
 * (gi_regular_grid_trilinear_function.h:285-341): per axis the products
 * kRKCoefficients[k][i] * f (float, src/gi_regular_grid_trilinear_function.cxx:5-11)
 * summed in double; k = min(1, distance to the boundary) (Gather1DNeighborhood,
 * gi_regular_grid.h:270-303), so the k = 0 row makes the component 0.0 + 0.0f*f. */
static double central_component(const float* f, int64_t idx, int64_t coord, int64_t n, int64_t stride) {
	static const float k1[3] = { -1.0f / 2.0f, 0.0f, 1.0f / 2.0f };
	int64_t dist = coord < (n - 1 - coord) ? coord : (n - 1 - coord);
	if (dist < 1) return 0.0 + (double)(0.0f * f[idx]);
	double r = 0.0;
	r += (double)(k1[0] * f[idx - stride]);
	r += (double)(k1[1] * f[idx]);
	r += (double)(k1[2] * f[idx + stride]);
	return r;
}

int oracle_central_diff_3d(const float* f, int64_t X, int64_t Y, int64_t Z, double* g) {
	if (X < 1 || Y < 1 || Z < 1) return -1;
	for (int64_t z = 0; z < Z; z++)
		for (int64_t y = 0; y < Y; y++)
			for (int64_t x = 0; x < X; x++) {
				int64_t v = x + X * (y + Y * z);
				g[3 * v + 0] = central_component(f, v, x, X, 1);
				g[3 * v + 1] = central_component(f, v, y, Y, X);
				g[3 * v + 2] = central_component(f, v, z, Z, X * Y);
			}
	return 0;
}

int oracle_central_diff_2d(const float* f, int64_t X, int64_t Y, double* g) {
	if (X < 1 || Y < 1) return -1;
	for (int64_t y = 0; y < Y; y++)
		for (int64_t x = 0; x < X; x++) {
			int64_t v = x + X * y;
			g[2 * v + 0] = central_component(f, v, x, X, 1);
			g[2 * v + 1] = central_component(f, v, y, Y, X);
		}
	return 0;
}


/* ---- Morse-Smale complex graph (MorseSmaleComplexBasic::ComputeFromGrad) ------------- */

typedef struct {
	const mesh_t* m;
	const uint8_t* g;
	const int64_t* node_cell;  /* critical cells, increasing */
	int64_t n_nodes;
	int64_t arc_cap, n_arcs;
	int32_t* lower;
	int32_t* upper;
	int64_t visits;  /* a .grad with a cycle (invalid input) would recurse forever */
	int depth, overflow;
} ms_trace_t;

/* nodeIdForCell (gi_morse_smale_complex_basic.h:212): the node of a critical cell */
static int64_t ms_node_of(const ms_trace_t* t, int64_t cell) {
	int64_t lo = 0, hi = t->n_nodes - 1;
	while (lo <= hi) {
		int64_t mid = (lo + hi) / 2;
		if (t->node_cell[mid] == cell) return mid;
		if (t->node_cell[mid] < cell) lo = mid + 1; else hi = mid - 1;
	}
	return -1;
}

/* rec_tdcr_candidates (gi_morse_smale_complex_basic.h:550-577): facets in order; a
 * critical facet ends a V-path (an arc to its node), a facet on the restricted
 * manifold (ldir == temp_dim) continues at its pair when that pair is another cell of
 * the traced cell's dimension. */
static void ms_trace_down(ms_trace_t* t, int64_t cell, int temp_dim, int32_t start) {
	int64_t c[3], fc[6];
	if (++t->visits > ((int64_t)1 << 26) || t->depth >= (1 << 14)) { t->overflow = 1; return; }
	cell_coords(t->m, cell, c);
	const int dim = cell_dim(t->m, c);
	const int nf = facets(t->m, cell, c, fc);
	for (int i = 0; i < nf; i++) {
		const uint8_t b = t->g[fc[i]];
		const uint8_t code = (uint8_t)((b & GB_PAIR_MSK) >> GB_PAIR_SH);
		if (code == 7) {
			const int64_t lower = ms_node_of(t, fc[i]);
			if (lower < 0) continue;
			if (t->n_arcs < t->arc_cap) {
				t->lower[t->n_arcs] = (int32_t)lower;
				t->upper[t->n_arcs] = start;
			}
			t->n_arcs++;
		} else if (code < 6 && (int)((b & GB_LDIR_MSK) >> GB_LDIR_SH) == temp_dim) {
			const int64_t p = decode_pair(t->m, fc[i], code);
			if (p < 0 || p >= t->m->ncells) continue;
			int64_t pc[3];
			cell_coords(t->m, p, pc);
			if (p != cell && cell_dim(t->m, pc) == dim) {
				t->depth++;
				ms_trace_down(t, p, temp_dim, start);
				t->depth--;
			}
		}
	}
}

int oracle_ms_graph_3d(const uint8_t* grad, const float* f, int64_t X, int64_t Y, int64_t Z, const int build[3],
                       int64_t node_cap, int64_t* node_cell, float* node_value, uint8_t* node_dim,
                       uint8_t* node_boundary, int64_t arc_cap, int32_t* arc_lower, int32_t* arc_upper,
                       float* arc_persistence, int64_t counts[2]) {
	mesh_t m;
	if (mesh_init(&m, 3, X, Y, Z)) return -1;
	/* the nodes: every critical cell, in AllCellsIterator (cell id) order */
	int64_t n = 0;
	for (int64_t i = 0; i < m.ncells; i++)
		if (((grad[i] & GB_PAIR_MSK) >> GB_PAIR_SH) == 7) n++;
	int64_t* cells = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
	float* val = (float*)malloc(sizeof(float) * (size_t)(n + 1));
	if (!cells || !val) { free(cells); free(val); return -2; }
	n = 0;
	for (int64_t i = 0; i < m.ncells; i++) {
		if (((grad[i] & GB_PAIR_MSK) >> GB_PAIR_SH) != 7) continue;
		int64_t c[3];
		cell_coords(&m, i, c);
		cells[n] = i;
		/* createNode: value = cellValue = f at Cell2HighestVertex */
		val[n] = f[extreme_vertex(&m, f, c, 1)];
		if (n < node_cap) {
			node_cell[n] = i;
			node_value[n] = val[n];
			node_dim[n] = (uint8_t)cell_dim(&m, c);
			node_boundary[n] = (uint8_t)boundary_value(&m, c);
		}
		n++;
	}
	/* the arcs: AddArcsThreadLocalNoGeom over the nodes in order (:600-620) */
	ms_trace_t t = { &m, grad, cells, n, arc_cap, 0, arc_lower, arc_upper, 0, 0, 0 };
	for (int64_t j = 0; j < n; j++) {
		int64_t c[3];
		cell_coords(&m, cells[j], c);
		const int d = cell_dim(&m, c);
		if (d == 0 || !build[d - 1]) continue;
		const int temp_dim = (int)((grad[cells[j]] & GB_LDIR_MSK) >> GB_LDIR_SH) + 1;
		const int64_t a0 = t.n_arcs;
		t.visits = 0;
		ms_trace_down(&t, cells[j], temp_dim, (int32_t)j);
		if (t.overflow) { free(cells); free(val); return -3; }
		for (int64_t a = a0; a < t.n_arcs && a < arc_cap; a++)
			if (arc_persistence) arc_persistence[a] = val[arc_upper[a]] - val[arc_lower[a]];
	}
	counts[0] = n;
	counts[1] = t.n_arcs;
	free(cells);
	free(val);
	return 0;
}
