// The C++ snippet of INTEGRATION.md (section 2), compiled against the MSCEER reference's
// own headers and sources: a reference program keeps its RegularGrid3D /
// RegularGridTrilinearFunction / TopologicalRegularGrid3D / DiscreteGradientLabeling
// objects and fills the labeling's byte array with one call of the C ABI, then writes
// the file with the reference's own writer.  Built by tests/test_integration_snippet.py.
//     integration_snippet X Y Z volume.raw out.grad
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "gi_discrete_gradient_labeling.h"
#include "gi_regular_grid.h"
#include "gi_regular_grid_trilinear_function.h"
#include "gi_topological_regular_grid.h"
#include "msc_gpu.h"

using namespace GInt;

int main(int argc, char** argv) {
  if (argc < 6) return 2;
  const int X = atoi(argv[1]), Y = atoi(argv[2]), Z = atoi(argv[3]);
  RegularGrid3D* grid = new RegularGrid3D(Vec3l(X, Y, Z), Vec3b(0, 0, 0));
  RegularGridTrilinearFunction* func = new RegularGridTrilinearFunction(grid);
  func->LoadImageFromFile(argv[4]);
  TopologicalRegularGrid3D* tgrid = new TopologicalRegularGrid3D(grid);
  typedef DiscreteGradientLabeling<TopologicalRegularGrid3D> GradType;

  // -- the snippet ----------------------------------------------------------------
  GradType* labeling = new GradType(tgrid);
  const int64_t dims[3] = {X, Y, Z};
  int rc = msc_steepest_lstar_host(func->GetImage(), dims, reinterpret_cast<uint8_t*>(labeling->m_dgrad->LabelArray()));
  if (rc != MSC_OK) {
    fprintf(stderr, "%s\n", msc_last_error_string());
    return 2;
  }
  labeling->outputToFile(argv[5]);
  // -------------------------------------------------------------------------------
  return 0;
}
