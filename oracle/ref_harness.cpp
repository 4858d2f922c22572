// Test-only harness: drives the reference MSCEER classes (compiled from the
// reference's own headers and src/*.cxx, see oracle/Makefile) and exposes them
// through a C ABI so the tests can pin the oracle restatement against the real
// reference.  Never linked into the product and never shipped to the GPU host.
//
// Pipelines reproduced (each step calls the reference class named):
//   ref_steepest_lstar_3d  == steepest_lstar/steepest_lstar.cxx:89-258
//       RegularGridMaxMinVertexLabeling3D::ComputeOutput   (gi_max_vertex_labeling.h:1119)
//       SlidingWindowRobinsNoalloc::ComputePairing_sliding (gi_fast_robins_noalloc.h:1254)
//       TopologicalGradientUsingAlgorithms::setAscendingManifoldDimensions
//                                                          (gi_topological_gradient_using_algorithms.h:430)
//       DiscreteGradientLabeling::outputToFile             (gi_discrete_gradient_labeling.h:200)
//   ref_lstar_grad_2d      == Accurate2D::DiscreteGradientBuilder::ComputeDiscreteGradient
//       without saddle streamlines (gi_discrete_gradient_computer.h:538-686)
//   ref_labels_3d[_threads] == ondemandaccurate/ondemandaccurate.cxx:795-948 (ASC and DSC
//       3-manifold labels); with a .grad path also the accurate .grad of :795-1063 with
//       needASC2 = needDSC2 = 1: VertexLabelingToBoundaryLabeling::ComputeMINBoundary /
//       ComputeMAXBoundary, the constrained MyRobinsNoalloc<...,4,6>::ComputeLowerStar of
//       the touched vertices and RecordGrad (:693-699)
//   ref_saddle_lines_3d    == ondemandaccurate/ondemandaccurate.cxx:254-505 at one thread
//       (in ref_harness_lines.cpp)
//   ref_ondemand_modes_3d  == ondemandaccurate/ondemandaccurate.cxx:772-1145 at one thread
//       for any of its needASC1 / needDSC1 / needASC2 / needDSC2 flags: the 3-manifold
//       labels and boundaries asked for, then the saddle lines on the gradient those
//       integrations left, then the re-pairing and RecordGrad
//   ref_ms_graph_3d        == extractmsc/extractmsc.cxx:482-504: a .grad loaded into
//       DiscreteGradientLabeling, LazyMaximumVertexLabeling + TopologicalMaxVertexMeshFunction,
//       MorseSmaleComplexBasic::ComputeFromGrad with the given arc build flags and no
//       arc geometry (gi_morse_smale_complex_basic.h:676-716)
//
// The only deviation from the shipped program: the mesh type is a thin subclass of
// TopologicalRegularGrid3D that adds a no-op cellid2Coords(INDEX_TYPE, Vec2l&)
// overload.  gi_modified_robins.h:1005-1013 builds an unused vector<Vec2l> through
// that overload, which the 3D mesh lacks, so the shipped headers do not compile for
// the 3D mesh.  The overload only feeds that dead vector; no algorithm step changes.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <queue>
#include <omp.h>

#include "gi_timing.h"
#include "gi_topological_explicit_mesh_function.h"
#include "gi_topological_gradient_using_algorithms.h"
#include "gi_topological_regular_grid_restricted.h"
#include "gi_topological_utility_functions.h"
#include "gi_numeric_integrator_expanding_region_stop.h"
#include "gi_topological_regular_masked_grid.h"
#include "gi_topological_regular_masked_restricted_grid.h"
#include "gi_max_vertex_labeling.h"
#include "gi_topological_max_vertex_mesh_function.h"
#include "gi_modified_robins.h"
#include "gi_fast_robins_noalloc.h"
#include "gi_discrete_gradient_computer.h"
#include "gi_extrema_region_builder.h"
#include "gi_numeric_integrator_path_compressing.h"
#include "gi_isolated_region_remover.h"
#include "gi_labeling_to_bounary_labeling.h"
#include "gi_morse_smale_complex_basic.h"

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

// the saddle loops of the needASC1 / needDSC1 modes (ref_harness_lines.cpp)
void saddle_lines(GridType* grid, GridFuncType* func, MeshType* mesh, GradType* labeling, TopoFuncType* topofunc,
                  DenseLabeling<char>* lab, int which, float error_threshold, float gradient_threshold,
                  int iteration_limit);

}  // namespace refharness

extern "C" {

// Runs the steepest_lstar pipeline on an in-memory float32 volume (x fastest) and
// writes the .grad file with the reference's own writer.  Returns 0 on success.
// stage_ms (optional, 3 doubles) receives max/min, Robins and ldir wall times.
int ref_steepest_lstar_3d(const float* f, long long X, long long Y, long long Z,
                          int nthreads, const char* grad_path, double* stage_ms) {
	using namespace refharness;
	if (nthreads > 0) omp_set_num_threads(nthreads);
	GridType* grid = new GridType(Vec3l(X, Y, Z), Vec3b(0, 0, 0));
	std::vector<float> img(f, f + X * Y * Z);
	GridFuncType* func = new GridFuncType(grid, img.data());
	MeshType* mesh = new MeshType(grid);

	auto t0 = std::chrono::steady_clock::now();
	MaxVLType* maxv = new MaxVLType(mesh, func);
	maxv->ComputeOutput();
	auto t1 = std::chrono::steady_clock::now();
	TopoFuncType* topofunc = new TopoFuncType();
	topofunc->setMeshAndFuncAndMaxVLabeling(mesh, func, maxv);
	GradType* labeling = new GradType(mesh);
	labeling->ClearAllGradient();
	NewRobinsType* robins = new NewRobinsType(grid, func, mesh, maxv, labeling);
	robins->ComputePairing_sliding();
	auto t2 = std::chrono::steady_clock::now();
	TopologicalGradientUsingAlgorithms<MeshType, TopoFuncType, GradType>* algs =
		new TopologicalGradientUsingAlgorithms<MeshType, TopoFuncType, GradType>(topofunc, mesh, labeling);
	algs->setAscendingManifoldDimensions();
	auto t3 = std::chrono::steady_clock::now();
	labeling->outputToFile(grad_path);
	if (stage_ms) {
		stage_ms[0] = std::chrono::duration<double, std::milli>(t1 - t0).count();
		stage_ms[1] = std::chrono::duration<double, std::milli>(t2 - t1).count();
		stage_ms[2] = std::chrono::duration<double, std::milli>(t3 - t2).count();
	}
	delete algs;
	delete robins;
	delete labeling;
	delete topofunc;
	delete maxv;
	delete mesh;
	delete func;
	delete grid;
	return 0;
}

// The 2D lower-star gradient of Accurate2D::DiscreteGradientBuilder with no saddle
// streamlines requested (gi_discrete_gradient_computer.h:561-583, 681-689).
int ref_lstar_grad_2d(const float* f, long long X, long long Y, int nthreads,
                      const char* grad_path, double* stage_ms) {
	using namespace Accurate2D;
	if (nthreads > 0) omp_set_num_threads(nthreads);
	GridType* grid = new GridType(Vec2i((int)X, (int)Y), Vec2b(0, 0));
	std::vector<float> img(f, f + X * Y);
	GridFuncType* func = new GridFuncType(grid, img.data());
	MeshType* mesh = new MeshType(grid);
	auto t0 = std::chrono::steady_clock::now();
	MaxVLType* maxv = new MaxVLType(mesh, func);
	maxv->ComputeOutput();
	auto t1 = std::chrono::steady_clock::now();
	MeshFuncType* topofunc = new MeshFuncType();
	topofunc->setMeshAndFuncAndMaxVLabeling(mesh, func, maxv);
	GradType* grad = new GradType(mesh);
	grad->ClearAllGradient();
	RobinsType* robins = new RobinsType(mesh, maxv, grad);
	robins->ComputePairing();
	auto t2 = std::chrono::steady_clock::now();
	TopologicalGradientUsingAlgorithms<MeshType, MeshFuncType, GradType>* algs =
		new TopologicalGradientUsingAlgorithms<MeshType, MeshFuncType, GradType>(topofunc, mesh, grad);
	algs->setAscendingManifoldDimensions();
	auto t3 = std::chrono::steady_clock::now();
	grad->outputToFile(grad_path);
	if (stage_ms) {
		stage_ms[0] = std::chrono::duration<double, std::milli>(t1 - t0).count();
		stage_ms[1] = std::chrono::duration<double, std::milli>(t2 - t1).count();
		stage_ms[2] = std::chrono::duration<double, std::milli>(t3 - t2).count();
	}
	delete algs;
	delete robins;
	delete grad;
	delete topofunc;
	delete maxv;
	delete mesh;
	delete func;
	delete grid;
	return 0;
}

// RegularGridTrilinearFunction::ComputeGradFromImage(1) on an in-memory volume;
// writes the Vec3d gradient array (3 doubles per vertex).
int ref_central_diff_3d(const float* f, long long X, long long Y, long long Z, double* out) {
	RegularGrid3D* grid = new RegularGrid3D(Vec3l(X, Y, Z), Vec3b(0, 0, 0));
	std::vector<float> img(f, f + X * Y * Z);
	RegularGridTrilinearFunction* func = new RegularGridTrilinearFunction(grid, img.data());
	func->ComputeGradFromImage(1);
	const long long n = X * Y * Z;
	for (long long v = 0; v < n; v++) {
		Vec3d gv = func->SampleGrad(Vec3l(v % X, (v / X) % Y, v / (X * Y)));
		out[3 * v + 0] = gv[0];
		out[3 * v + 1] = gv[1];
		out[3 * v + 2] = gv[2];
	}
	delete func;
	delete grid;
	return 0;
}

// ondemandaccurate's ASC and DSC 3-manifold labels (ondemandaccurate.cxx:795-948)
// with one OpenMP thread, which makes the reference deterministic.  Labels are the
// reference's unique-id numbers mapped to the smallest seed vertex of their region
// (the reference draws the numbers from unordered_map order).  stage (optional, 4*N):
// terminal and integrated labels, ASC then DSC, mapped the same way.
int ref_ondemand_3d(const float* f, long long X, long long Y, long long Z, float error_threshold,
                    float gradient_threshold, int iteration_limit, float presimp, int* asc, int* dsc, int* stage,
                    int nthreads, const char* grad_path, unsigned char* restrict_out);
int ref_labels_3d(const float* f, long long X, long long Y, long long Z, float error_threshold,
                  float gradient_threshold, int iteration_limit, float presimp, int* asc, int* dsc, int* stage) {
	return ref_ondemand_3d(f, X, Y, Z, error_threshold, gradient_threshold, iteration_limit, presimp, asc, dsc, stage,
	                       1, nullptr, nullptr);
}

// The same at `nthreads` OpenMP threads: the reference's own run-to-run / thread-count
// variation of the labels (its parallel first pass and fix-up race) is the yardstick
// of the label tolerances.
int ref_labels_3d_threads(const float* f, long long X, long long Y, long long Z, float error_threshold,
                          float gradient_threshold, int iteration_limit, float presimp, int* asc, int* dsc,
                          int* stage, int nthreads) {
	return ref_ondemand_3d(f, X, Y, Z, error_threshold, gradient_threshold, iteration_limit, presimp, asc, dsc, stage,
	                       nthreads, nullptr, nullptr);
}

// With grad_path: also the accurate .grad ondemandaccurate writes for needASC2 =
// needDSC2 = 1 (and, optionally, the restriction labels, one byte per cell).
int ref_ondemand_3d(const float* f, long long X, long long Y, long long Z, float error_threshold,
                    float gradient_threshold, int iteration_limit, float presimp, int* asc, int* dsc, int* stage,
                    int nthreads, const char* grad_path, unsigned char* restrict_out) {
	using namespace refharness;
	typedef IndexCompareLessThan<GridFuncType> ComparerASC;
	typedef IndexCompareGreaterThan<GridFuncType> ComparerDSC;
	typedef NumericIntegratorPathCompressingToTerminal<AdaptiveEulerAdvector3D<GridFuncType, -1>, GridFuncType> IntASC;
	typedef NumericIntegratorPathCompressingToTerminal<AdaptiveEulerAdvector3D<GridFuncType, 1>, GridFuncType> IntDSC;
	omp_set_num_threads(nthreads > 0 ? nthreads : 1);
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
	SimplifiedExtremumGraph<MeshType, TopoFuncType, GradType>* seg =
		new SimplifiedExtremumGraph<MeshType, TopoFuncType, GradType>(mesh, topofunc, labeling);
	seg->SetMode(SimplifiedExtremumGraph<MeshType, TopoFuncType, GradType>::EXTGRAPHMODE::BOTH);
	seg->ComputeMinMapFromGradient(presimp);
	const long long N = X * Y * Z;
	DenseLabeling<char>* restriction_labels = new DenseLabeling<char>(mesh->numCells());
	restriction_labels->SetAll(0);
	VertexLabelingToBoundaryLabeling<int, MaxVLType>* edge_map =
		new VertexLabelingToBoundaryLabeling<int, MaxVLType>(mesh, restriction_labels);
	edge_map->InitializeFirst();

	auto canon = [&](const std::unordered_map<INT_TYPE, std::vector<INDEX_TYPE> >& idmap, DenseLabeling<int>* terminal) {
		std::unordered_map<int, long long> c;
		for (auto& kv : idmap) {
			long long mn = -1;
			for (auto v : kv.second) if (mn < 0 || v < mn) mn = v;
			c[terminal->GetLabel(kv.second[0])] = mn;
		}
		return c;
	};
	auto write = [&](int* out, DenseLabeling<int>* lab, std::unordered_map<int, long long>& c) {
		for (long long v = 0; v < N; v++) {
			int l = lab->GetLabel(v);
			out[v] = (l < 0) ? -1 : (int)c[l];
		}
	};

	{
		std::unordered_map<INDEX_TYPE, INT_TYPE> ext;
		for (auto p : seg->mMinGraph->mCellIndexToListIdMap) ext[p.first] = seg->mMinGraph->Representative(p.second);
		GridSimplifiedExtremalRegionBuilder<ComparerASC, GridFuncType, MeshType>* rb =
			new GridSimplifiedExtremalRegionBuilder<ComparerASC, GridFuncType, MeshType>(func, grid, mesh);
		rb->BeginIntegration(ext);
		auto c = canon(rb->GetIdMap(), rb->GetOutputLabels());
		if (stage) write(stage, rb->GetOutputLabels(), c);
		IntASC* integ = new IntASC(func, grid, error_threshold, gradient_threshold, iteration_limit);
		integ->BeginIntegration(rb->GetIdMap(), rb->GetOutputLabels(), false);
		if (stage) write(stage + N, integ->GetOutputLabels(), c);
		IsolatedCCRegionRemoverNEW<ComparerASC, GridFuncType>* cl =
			new IsolatedCCRegionRemoverNEW<ComparerASC, GridFuncType>(func, integ->GetOutputLabels());
		cl->ComputeOutput();
		write(asc, integ->GetOutputLabels(), c);
		if (grad_path) edge_map->ComputeMINBoundary(integ->GetOutputLabels());
	}
	{
		std::unordered_map<INDEX_TYPE, INT_TYPE> ext;
		for (auto p : seg->mMaxGraph->mCellIndexToListIdMap)
			ext[maxv->Cell2HighestVertex(p.first)] = seg->mMaxGraph->Representative(p.second);
		GridSimplifiedExtremalRegionBuilder<ComparerDSC, GridFuncType, MeshType>* rb =
			new GridSimplifiedExtremalRegionBuilder<ComparerDSC, GridFuncType, MeshType>(func, grid, mesh);
		rb->BeginIntegration(ext);
		auto c = canon(rb->GetIdMap(), rb->GetOutputLabels());
		if (stage) write(stage + 2 * N, rb->GetOutputLabels(), c);
		IntDSC* integ = new IntDSC(func, grid, error_threshold, gradient_threshold, iteration_limit);
		integ->BeginIntegration(rb->GetIdMap(), rb->GetOutputLabels(), false);
		if (stage) write(stage + 3 * N, integ->GetOutputLabels(), c);
		IsolatedCCRegionRemoverNEW<ComparerDSC, GridFuncType>* cl =
			new IsolatedCCRegionRemoverNEW<ComparerDSC, GridFuncType>(func, integ->GetOutputLabels());
		cl->ComputeOutput();
		write(dsc, integ->GetOutputLabels(), c);
		if (grad_path) edge_map->ComputeMAXBoundary(integ->GetOutputLabels(), maxv);
	}
	if (grad_path) {
		// ondemandaccurate.cxx:1000-1063 (one thread): re-pair every vertex that is
		// restricted or whose lower star holds a restricted cell, then RecordGrad
		typedef MyRobinsNoalloc<MeshType, MaxVLType, GradType, 4, 6> RobinsType;
		RobinsType* constrained = new RobinsType(mesh, maxv, restriction_labels, labeling);
		MeshType::DCellsIterator verts(mesh, 0);
		for (verts.begin(); verts.valid(); verts.advance()) {
			INDEX_TYPE vert_GI = verts.value();
			bool hasdiff = restriction_labels->GetLabel(vert_GI) > 0;
			if (!hasdiff) {
				MeshType::AdjacentCellsIterator edgeit(mesh);
				for (edgeit.begin(vert_GI); edgeit.valid(); edgeit.advance()) {
					INDEX_TYPE edge_GI = edgeit.value();
					if (restriction_labels->GetLabel(edge_GI) > 0 && maxv->Cell2HighestVertex(edge_GI) == vert_GI) {
						hasdiff = true;
						break;
					}
				}
			}
			if (hasdiff) constrained->ComputeLowerStar(vert_GI);
		}
		TopologicalGradientUsingAlgorithms<MeshType, TopoFuncType, GradType>* alg =
			new TopologicalGradientUsingAlgorithms<MeshType, TopoFuncType, GradType>(topofunc, mesh, labeling);
		alg->setAscendingManifoldDimensions();
		labeling->outputToFile(grad_path);
		if (restrict_out)
			for (long long i = 0; i < (long long)mesh->numCells(); i++) restrict_out[i] = (unsigned char)restriction_labels->GetLabel(i);
	}
	return 0;   // the reference objects are left to the process (their destructors double-free shared labels)
}


// Nodes (cell, value, dim, boundary) and arcs (lower, upper, persistence) of
// MorseSmaleComplexBasic::ComputeFromGrad on a finished .grad; counts[0] nodes,
// counts[1] arcs, arrays filled up to their caps.
int ref_ms_graph_3d(const float* f, long long X, long long Y, long long Z, const unsigned char* grad, const int* build,
                    int nthreads, long long node_cap, long long* node_cell, float* node_value, unsigned char* node_dim,
                    unsigned char* node_boundary, long long arc_cap, int* arc_lower, int* arc_upper,
                    float* arc_persistence, long long* counts) {
	using namespace refharness;
	typedef LazyMaximumVertexLabeling<MeshType, GridFuncType> LazyMaxVLType;
	typedef TopologicalMaxVertexMeshFunction<MeshType, LazyMaxVLType, GridFuncType, float> LazyTopoFuncType;
	typedef MorseSmaleComplexBasic<float, MeshType, LazyTopoFuncType, GradType> MscType;
	if (nthreads > 0) omp_set_num_threads(nthreads);
	GridType* grid = new GridType(Vec3l(X, Y, Z), Vec3b(0, 0, 0));
	std::vector<float> img(f, f + X * Y * Z);
	GridFuncType* func = new GridFuncType(grid, img.data());
	MeshType* mesh = new MeshType(grid);
	LazyMaxVLType* maxv = new LazyMaxVLType(mesh, func);
	maxv->ComputeOutput();
	LazyTopoFuncType* topofunc = new LazyTopoFuncType();
	topofunc->setMeshAndFuncAndMaxVLabeling(mesh, func, maxv);
	GradType* labeling = new GradType(mesh);
	std::memcpy(labeling->m_dgrad->LabelArray(), grad, (size_t)mesh->numCells());
	MscType* msc = new MscType(labeling, mesh, topofunc);
	msc->SetBuildArcGeometry(Vec3b(false, false, false));
	msc->SetBuildArcs(Vec3b(build[0] != 0, build[1] != 0, build[2] != 0));
	msc->ComputeFromGrad();
	const long long nn = msc->numNodes(), na = msc->numArcs();
	for (long long i = 0; i < nn && i < node_cap; i++) {
		const auto& n = msc->getNode((INT_TYPE)i);
		node_cell[i] = (long long)n.cellindex;
		node_value[i] = n.value;
		node_dim[i] = (unsigned char)n.dim;
		node_boundary[i] = (unsigned char)n.boundary;
	}
	for (long long i = 0; i < na && i < arc_cap; i++) {
		const auto& a = msc->getArc((INT_TYPE)i);
		arc_lower[i] = (int)a.lower;
		arc_upper[i] = (int)a.upper;
		arc_persistence[i] = a.persistence;
	}
	counts[0] = nn;
	counts[1] = na;
	return 0;   // the reference objects are left to the process, as above
}

// ondemandaccurate's accurate .grad for the flags a1 d1 a2 d2 (needASC1, needDSC1,
// needASC2, needDSC2) at one thread, with its restriction labels (one byte per cell).
int ref_ondemand_modes_3d(const float* f, long long X, long long Y, long long Z, float error_threshold,
                          float gradient_threshold, int iteration_limit, float presimp, int a1, int d1, int a2, int d2,
                          const char* grad_path, unsigned char* restrict_out) {
	using namespace refharness;
	typedef IndexCompareLessThan<GridFuncType> ComparerASC;
	typedef IndexCompareGreaterThan<GridFuncType> ComparerDSC;
	typedef NumericIntegratorPathCompressingToTerminal<AdaptiveEulerAdvector3D<GridFuncType, -1>, GridFuncType> IntASC;
	typedef NumericIntegratorPathCompressingToTerminal<AdaptiveEulerAdvector3D<GridFuncType, 1>, GridFuncType> IntDSC;
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
	DenseLabeling<char>* restriction_labels = new DenseLabeling<char>(mesh->numCells());
	restriction_labels->SetAll(0);
	if (a1 || d1 || a2 || d2) {
		func->ComputeGradFromImage(1);
		if (a2 || d2) {
			SimplifiedExtremumGraph<MeshType, TopoFuncType, GradType>* seg =
				new SimplifiedExtremumGraph<MeshType, TopoFuncType, GradType>(mesh, topofunc, labeling);
			seg->SetMode(a2 && d2 ? SimplifiedExtremumGraph<MeshType, TopoFuncType, GradType>::EXTGRAPHMODE::BOTH
			             : a2 ? SimplifiedExtremumGraph<MeshType, TopoFuncType, GradType>::EXTGRAPHMODE::MINS
			                  : SimplifiedExtremumGraph<MeshType, TopoFuncType, GradType>::EXTGRAPHMODE::MAXS);
			seg->ComputeMinMapFromGradient(presimp);
			VertexLabelingToBoundaryLabeling<int, MaxVLType>* edge_map =
				new VertexLabelingToBoundaryLabeling<int, MaxVLType>(mesh, restriction_labels);
			edge_map->InitializeFirst();
			if (a2) {
				std::unordered_map<INDEX_TYPE, INT_TYPE> ext;
				for (auto p : seg->mMinGraph->mCellIndexToListIdMap) ext[p.first] = seg->mMinGraph->Representative(p.second);
				GridSimplifiedExtremalRegionBuilder<ComparerASC, GridFuncType, MeshType>* rb =
					new GridSimplifiedExtremalRegionBuilder<ComparerASC, GridFuncType, MeshType>(func, grid, mesh);
				rb->BeginIntegration(ext);
				IntASC* integ = new IntASC(func, grid, error_threshold, gradient_threshold, iteration_limit);
				integ->BeginIntegration(rb->GetIdMap(), rb->GetOutputLabels(), false);
				IsolatedCCRegionRemoverNEW<ComparerASC, GridFuncType>* cl =
					new IsolatedCCRegionRemoverNEW<ComparerASC, GridFuncType>(func, integ->GetOutputLabels());
				cl->ComputeOutput();
				edge_map->ComputeMINBoundary(integ->GetOutputLabels());
			}
			if (d2) {
				std::unordered_map<INDEX_TYPE, INT_TYPE> ext;
				for (auto p : seg->mMaxGraph->mCellIndexToListIdMap)
					ext[maxv->Cell2HighestVertex(p.first)] = seg->mMaxGraph->Representative(p.second);
				GridSimplifiedExtremalRegionBuilder<ComparerDSC, GridFuncType, MeshType>* rb =
					new GridSimplifiedExtremalRegionBuilder<ComparerDSC, GridFuncType, MeshType>(func, grid, mesh);
				rb->BeginIntegration(ext);
				IntDSC* integ = new IntDSC(func, grid, error_threshold, gradient_threshold, iteration_limit);
				integ->BeginIntegration(rb->GetIdMap(), rb->GetOutputLabels(), false);
				IsolatedCCRegionRemoverNEW<ComparerDSC, GridFuncType>* cl =
					new IsolatedCCRegionRemoverNEW<ComparerDSC, GridFuncType>(func, integ->GetOutputLabels());
				cl->ComputeOutput();
				edge_map->ComputeMAXBoundary(integ->GetOutputLabels(), maxv);
			}
		}
		if (a1 || d1)
			saddle_lines(grid, func, mesh, labeling, topofunc, restriction_labels, (a1 ? 1 : 0) | (d1 ? 2 : 0),
			             error_threshold, gradient_threshold, iteration_limit);
		typedef MyRobinsNoalloc<MeshType, MaxVLType, GradType, 4, 6> RobinsType;
		RobinsType* constrained = new RobinsType(mesh, maxv, restriction_labels, labeling);
		MeshType::DCellsIterator verts(mesh, 0);
		for (verts.begin(); verts.valid(); verts.advance()) {
			INDEX_TYPE vert_GI = verts.value();
			bool hasdiff = restriction_labels->GetLabel(vert_GI) > 0;
			if (!hasdiff) {
				MeshType::AdjacentCellsIterator cells(mesh);
				for (cells.begin(vert_GI); cells.valid(); cells.advance()) {
					INDEX_TYPE cell_GI = cells.value();
					if (restriction_labels->GetLabel(cell_GI) > 0 && maxv->Cell2HighestVertex(cell_GI) == vert_GI) {
						hasdiff = true;
						break;
					}
				}
			}
			if (hasdiff) constrained->ComputeLowerStar(vert_GI);
		}
	}
	TopologicalGradientUsingAlgorithms<MeshType, TopoFuncType, GradType>* alg =
		new TopologicalGradientUsingAlgorithms<MeshType, TopoFuncType, GradType>(topofunc, mesh, labeling);
	alg->setAscendingManifoldDimensions();
	labeling->outputToFile(grad_path);
	if (restrict_out)
		for (long long i = 0; i < (long long)mesh->numCells(); i++) restrict_out[i] = (unsigned char)restriction_labels->GetLabel(i);
	return 0;   // the reference objects are left to the process, as above
}

}  // extern "C"
