// Test-only harness, second translation unit: the saddle streamline digitizers of
// ondemandaccurate's needASC1 / needDSC1 modes, driven through the reference's own
// classes (see ref_harness.cpp for the setup the two files share).
//
//   ref_saddle_lines_3d == ondemandaccurate/ondemandaccurate.cxx:254-505 at one thread
//       (ReIntegrateUpFrom2Saddles / ReIntegrateDownFrom1Saddles: the saddle loop written
//       out here, single-threaded, around the reference's DigitizingNumericStreamline-
//       Integrator3dASC / 3dDSC, gi_numeric_streamline_integrator.h:525-1080, with the
//       gradient ComputeGradFromImage(1) of f and the targets 4 / 5 of :1075-1090)
//
// This file is compiled apart (oracle/Makefile): DigitizeSegmentInternal
// (gi_numeric_streamline_integrator.h:558-713) can flow off the end of a function that
// returns a value, whose value its caller ignores.  GCC turns that end into a trap at -O0
// and into unreachable code with optimisation (the harness then crashed); built with
// -O0 -fno-unreachable-traps the function returns as the program intends.  The
// floating point is the same at every level on x86-64 (SSE2, no fused multiply-add).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <queue>
#include <omp.h>

#include "gi_timing.h"
#include "gi_topological_gradient_using_algorithms.h"
#include "gi_max_vertex_labeling.h"
#include "gi_topological_max_vertex_mesh_function.h"
#include "gi_modified_robins.h"
#include "gi_fast_robins_noalloc.h"
#include "gi_numeric_streamline_integrator.h"
#include <algorithm>
#include <set>

using namespace GInt;

namespace refharness {

class Mesh3D : public TopologicalRegularGrid3D {
public:
	explicit Mesh3D(RegularGrid3D* g) : TopologicalRegularGrid3D(g) {}
	using TopologicalRegularGrid3D::cellid2Coords;
	// feeds only the unused vector at gi_modified_robins.h:1005-1013
	inline void cellid2Coords(INDEX_TYPE, Vec2l& c) const { c[0] = 0; c[1] = 0; }
};

typedef RegularGrid3D GridType;
typedef RegularGridTrilinearFunction GridFuncType;
typedef Mesh3D MeshType;
typedef DiscreteGradientLabeling<MeshType> GradType;
typedef RegularGridMaxMinVertexLabeling3D<MeshType, GridFuncType> MaxVLType;
typedef TopologicalMaxVertexMeshFunction<MeshType, MaxVLType, GridFuncType, float> TopoFuncType;
typedef SlidingWindowRobinsNoalloc<GridType, GridFuncType, MeshType, MaxVLType, GradType> NewRobinsType;

}  // namespace refharness

namespace refharness {

// The saddle loops of ReIntegrateUpFrom2Saddles (which bit 0, label 4) and
// ReIntegrateDownFrom1Saddles (bit 1, label 5) at one thread, on the given objects.
void saddle_lines(GridType* grid, GridFuncType* func, MeshType* mesh, GradType* labeling, TopoFuncType* topofunc,
                  DenseLabeling<char>* lab, int which, float error_threshold, float gradient_threshold,
                  int iteration_limit) {
	typedef DigitizingNumericStreamlineIntegrator3dASC<MeshType, GridFuncType, AdaptiveEulerAdvector3D<GridFuncType, 1> >
		DigASC;
	typedef DigitizingNumericStreamlineIntegrator3dDSC<MeshType, GridFuncType, AdaptiveEulerAdvector3D<GridFuncType, -1> >
		DigDSC;
	// the saddles of dimension sdim by the reference's keys, the last processed first
	auto saddles = [&](int sdim, bool negate) {
		std::vector<std::pair<float, INDEX_TYPE> > cr;
		MeshType::DCellsIterator it(mesh, sdim);
		for (it.begin(); it.valid(); it.advance()) {
			const INDEX_TYPE id = it.value();
			if (!labeling->getCritical(id)) continue;
			const float v = topofunc->cellValue(id);
			cr.push_back(std::pair<float, INDEX_TYPE>(negate ? -1 * v : v, id));
		}
		std::sort(cr.begin(), cr.end());
		return cr;
	};
	// the cells around a saddle its streamlines start from: a breadth-first walk of at
	// most five cells through the cofacets (up) or facets (down) and their pairs
	auto around = [&](INDEX_TYPE sad, bool up) {
		std::vector<INDEX_TYPE> result;
		std::queue<INDEX_TYPE> q;
		std::set<INDEX_TYPE> seen;
		q.push(sad);
		for (int counter = 4; !q.empty() && counter >= 0; counter--) {
			const INDEX_TYPE cur = q.front();
			q.pop();
			seen.insert(cur);
			std::vector<INDEX_TYPE> next;
			if (up) {
				MeshType::CofacetsIterator cf(mesh);
				for (cf.begin(cur); cf.valid(); cf.advance()) next.push_back(cf.value());
			} else {
				MeshType::FacetsIterator fc(mesh);
				for (fc.begin(cur); fc.valid(); fc.advance()) next.push_back(fc.value());
			}
			for (INDEX_TYPE t : next) {
				if (seen.count(t)) continue;
				result.push_back(t);
				seen.insert(t);
				if (!labeling->getCritical(t)) {
					const INDEX_TYPE p = labeling->getPair(t);
					seen.insert(p);
					q.push(p);
				}
			}
		}
		return result;
	};
	if (which & 1) {
		DigASC* dig = new DigASC(grid, func, mesh, error_threshold, gradient_threshold, iteration_limit);
		dig->SetDigitizingTarget(lab, 4);
		auto cr = saddles(2, false);
		for (long long li = (long long)cr.size() - 1; li >= 0; li--) {
			for (INDEX_TYPE h : around(cr[li].second, true)) {
				if (mesh->dimension(h) != 3) continue;
				std::vector<Vec3d> points;
				std::vector<INDEX_TYPE> dline;
				Vec3d seed;
				mesh->centroid(h, seed);
				seed = seed * 0.5;
				dig->IntegrateStreamline(seed, points, dline);
			}
			dig->set_label(cr[li].second);
		}
	}
	if (which & 2) {
		DigDSC* dig = new DigDSC(grid, func, mesh, error_threshold, gradient_threshold, iteration_limit);
		dig->SetDigitizingTarget(lab, 5);
		auto cr = saddles(1, true);
		for (long long li = (long long)cr.size() - 1; li >= 0; li--) {
			for (INDEX_TYPE v : around(cr[li].second, false)) {
				if (mesh->dimension(v) != 0) continue;
				std::vector<Vec3d> points;
				std::vector<INDEX_TYPE> dline;
				Vec3d seed;
				mesh->centroid(v, seed);
				seed = seed * 0.5;
				dig->IntegrateStreamline(seed, points, dline);
			}
			dig->set_label(cr[li].second);
		}
	}
}

}  // namespace refharness

extern "C" {

// The saddle streamline digitizers at one thread on the gradient of f: which bit 0 the
// ascending lines from the 2-saddles (label 4), bit 1 the descending lines from the
// 1-saddles (label 5), in that order, into cells (one byte per cell, in and out).
int ref_saddle_lines_3d(const float* f, long long X, long long Y, long long Z, int which, float error_threshold,
                        float gradient_threshold, int iteration_limit, unsigned char* cells) {
	using namespace refharness;
	omp_set_num_threads(1);
	GridType* grid = new GridType(Vec3l(X, Y, Z), Vec3b(0, 0, 0));
	std::vector<float> img(f, f + X * Y * Z);
	GridFuncType* func = new GridFuncType(grid, img.data());
	MeshType* mesh = new MeshType(grid);
	MaxVLType* maxv = new MaxVLType(mesh, func);
	maxv->ComputeOutput();
	TopoFuncType* topofunc = new TopoFuncType();
	topofunc->setMeshAndFuncAndMaxVLabeling(mesh, func, maxv);
	GradType* labeling = new GradType(mesh);
	labeling->ClearAllGradient();
	NewRobinsType* robins = new NewRobinsType(grid, func, mesh, maxv, labeling);
	robins->ComputePairing_sliding();
	func->ComputeGradFromImage(1);
	const INDEX_TYPE NC = mesh->numCells();
	DenseLabeling<char>* lab = new DenseLabeling<char>(NC);
	for (INDEX_TYPE i = 0; i < NC; i++) lab->SetLabel(i, (char)cells[i]);

	saddle_lines(grid, func, mesh, labeling, topofunc, lab, which, error_threshold, gradient_threshold, iteration_limit);
	for (INDEX_TYPE i = 0; i < NC; i++) cells[i] = (unsigned char)lab->GetLabel(i);
	return 0;   // the reference objects are left to the process, as above
}

}  // extern "C"
