// The Morse-Smale complex snippet of INTEGRATION.md (section 2), compiled against the
// MSCEER reference's own headers: an extractmsc-style program loads a .grad, calls
// msc_ms_graph_3d for the node and arc arrays, and builds the reference's
// MorseSmaleComplexBasic from them; the program then checks that object against the
// reference's own ComputeFromGrad on the same .grad.  Built by
// tests/test_integration_snippet.py, with the library call served by a CPU stand-in.
//     integration_ms_graph X Y Z volume.raw volume.grad
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

// the include list of extractmsc/extractmsc.h
#include "gi_basic_types.h"
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
#include "gi_morse_smale_complex_basic.h"
#include "msc_gpu.h"

using namespace GInt;

typedef TopologicalRegularGrid3D MeshType;
typedef RegularGridTrilinearFunction GridFuncType;
typedef DiscreteGradientLabeling<MeshType> GradType;
typedef LazyMaximumVertexLabeling<MeshType, GridFuncType> MaxVLType;
typedef TopologicalMaxVertexMeshFunction<MeshType, MaxVLType, GridFuncType, float> TopoFuncType;
typedef MorseSmaleComplexBasic<float, MeshType, TopoFuncType, GradType> MscType;

// -- the snippet --------------------------------------------------------------------
// The node and arc creators of MorseSmaleComplexBasic are protected: a subclass fills
// the complex from the library's arrays (copied to the host).
class DeviceGraphMsc : public MscType {
 public:
  using MscType::MscType;
  void FromArrays(int64_t n, const int64_t* cell, const float* value, int64_t na, const int32_t* lower,
                  const int32_t* upper) {
    for (int64_t i = 0; i < n; i++) createNode((INDEX_TYPE)cell[i], value[i]);
    for (int64_t a = 0; a < na; a++) createArcFromNodeIDs(lower[a], upper[a]);
  }
};
// -----------------------------------------------------------------------------------

int main(int argc, char** argv) {
  if (argc < 6) return 2;
  const int X = atoi(argv[1]), Y = atoi(argv[2]), Z = atoi(argv[3]);
  RegularGrid3D* grid = new RegularGrid3D(Vec3l(X, Y, Z), Vec3b(0, 0, 0));
  GridFuncType* func = new GridFuncType(grid);
  func->LoadImageFromFile(argv[4]);
  MeshType* mesh = new MeshType(grid);
  MaxVLType* maxv = new MaxVLType(mesh, func);
  maxv->ComputeOutput();
  TopoFuncType* topo = new TopoFuncType();
  topo->setMeshAndFuncAndMaxVLabeling(mesh, func, maxv);
  GradType* grad = new GradType(mesh);
  grad->load_from_file(argv[5]);

  // -- the snippet ------------------------------------------------------------------
  const int64_t dims[3] = {X, Y, Z};
  const int build[3] = {1, 0, 1};  // extractmsc: no saddle-saddle arcs
  int64_t counts[2];
  // grad_dev / f_dev: the .grad and the image in device memory (here the stand-in
  // library reads host memory)
  const uint8_t* grad_dev = reinterpret_cast<const uint8_t*>(grad->m_dgrad->LabelArray());
  const float* f_dev = func->GetImage();
  if (msc_ms_graph_3d(grad_dev, f_dev, dims, build, 0, nullptr, nullptr, nullptr, nullptr, 0, nullptr, nullptr,
                      nullptr, counts, nullptr) != MSC_OK)
    return 3;
  std::vector<int64_t> cell(counts[0]);
  std::vector<float> value(counts[0]);
  std::vector<uint8_t> ndim(counts[0]), nbnd(counts[0]);
  std::vector<int32_t> lower(counts[1]), upper(counts[1]);
  if (msc_ms_graph_3d(grad_dev, f_dev, dims, build, counts[0], cell.data(), value.data(), ndim.data(), nbnd.data(),
                      counts[1], lower.data(), upper.data(), nullptr, counts, nullptr) != MSC_OK)
    return 3;
  DeviceGraphMsc* msc = new DeviceGraphMsc(grad, mesh, topo);
  msc->FromArrays(counts[0], cell.data(), value.data(), counts[1], lower.data(), upper.data());
  // -----------------------------------------------------------------------------------

  MscType* ref = new MscType(grad, mesh, topo);
  ref->SetBuildArcGeometry(Vec3b(false, false, false));
  ref->SetBuildArcs(Vec3b(true, false, true));
  ref->ComputeFromGrad();
  if (ref->numNodes() != msc->numNodes() || ref->numArcs() != msc->numArcs()) return 4;
  for (INT_TYPE i = 0; i < ref->numNodes(); i++) {
    const auto &a = ref->getNode(i), &b = msc->getNode(i);
    if (a.cellindex != b.cellindex || a.dim != b.dim || a.boundary != b.boundary || a.value != b.value ||
        a.numarcs != b.numarcs || a.numlower != b.numlower || a.firstarc != b.firstarc)
      return 5;
  }
  for (INT_TYPE i = 0; i < ref->numArcs(); i++) {
    const auto &a = ref->getArc(i), &b = msc->getArc(i);
    if (a.lower != b.lower || a.upper != b.upper || a.persistence != b.persistence || a.dim != b.dim ||
        a.lower_next != b.lower_next || a.upper_next != b.upper_next)
      return 6;
  }
  printf("%lld nodes %lld arcs equal\n", (long long)ref->numNodes(), (long long)ref->numArcs());
  return 0;
}
