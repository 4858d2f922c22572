// steepest_lstar -- drop-in for MSCEER's steepest_lstar/steepest_lstar.cxx on one GB300.
//
// Same command line (steepest_lstar.cxx:61-72):
//     steepest_lstar X Y Z filename per_x per_y per_z [numthreads]
// reads X*Y*Z float32 (x fastest) from `filename` and writes `filename.grad`, one
// GradBitfield byte per cell, bit-identical to the reference's output, plus the
// `filename.steep.gtime.txt` timing line (steepest_lstar.cxx:100-101,217-220).
// As in the reference the mesh is always non-periodic (per_* are parsed and
// ignored, steepest_lstar.cxx:111) and numthreads is accepted and ignored (the
// work runs on the GPU).  Exit status mirrors the reference: 0 after the usage
// message, 1 after a completed run; a failure prints the library error and
// returns 2.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "msc_gpu.h"

int main(int argc, char** argv) {
  if (argc < 8) {
    printf("Usage: X Y Z filename per_x per_y per_z  [numthreads=max_on_machine]\n");
    return 0;
  }
  int X = 0, Y = 0, Z = 0, per_x = 0, per_y = 0, per_z = 0, numthreads = 0;
  sscanf(argv[1], "%d", &X);
  sscanf(argv[2], "%d", &Y);
  sscanf(argv[3], "%d", &Z);
  std::string filename(argv[4]);
  sscanf(argv[5], "%d", &per_x);
  sscanf(argv[6], "%d", &per_y);
  sscanf(argv[7], "%d", &per_z);
  if (argc >= 9) sscanf(argv[8], "%d", &numthreads);
  printf("%d, %d, %d, %d, %d, %d, %d\n", X, Y, Z, per_x, per_y, per_z, numthreads);

  const int64_t dims[3] = {X, Y, Z};
  const int64_t ncells = msc_num_cells_3d(dims);
  if (ncells < 0) {
    fprintf(stderr, "steepest_lstar: invalid dimensions %d %d %d\n", X, Y, Z);
    return 2;
  }
  const size_t nv = (size_t)X * (size_t)Y * (size_t)Z;
  std::vector<float> f(nv);
  FILE* fin = fopen(filename.c_str(), "rb");
  if (!fin) {
    fprintf(stderr, "steepest_lstar: cannot open %s\n", filename.c_str());
    return 2;
  }
  size_t got = fread(f.data(), sizeof(float), nv, fin);
  fclose(fin);
  if (got != nv) {
    fprintf(stderr, "steepest_lstar: %s holds %zu of %zu values\n", filename.c_str(), got, nv);
    return 2;
  }
  printf("loaded cont function\n");

  auto t0 = std::chrono::steady_clock::now();
  std::vector<uint8_t> grad((size_t)ncells);
  int rc = msc_steepest_lstar_host(f.data(), dims, grad.data());
  auto t1 = std::chrono::steady_clock::now();
  if (rc != MSC_OK) {
    fprintf(stderr, "steepest_lstar: %s (status %d)\n", msc_last_error_string(), rc);
    return 2;
  }
  const long long ms = std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count();
  std::string tname = filename + ".steep.gtime.txt";
  if (FILE* gt = fopen(tname.c_str(), "w")) {
    fprintf(gt, "Total Overall %d %lld %lld\n", 0, ms, ms);
    fclose(gt);
  }
  printf("Total Overall %d %lld %lld\n", 0, ms, ms);

  std::string gname = filename + ".grad";
  FILE* fg = fopen(gname.c_str(), "wb");
  if (!fg) {
    fprintf(stderr, "steepest_lstar: cannot write %s\n", gname.c_str());
    return 2;
  }
  printf("Going to output %lld cells in %s...\n", (long long)ncells, gname.c_str());
  size_t put = fwrite(grad.data(), 1, grad.size(), fg);
  fclose(fg);
  if (put != grad.size()) {
    fprintf(stderr, "steepest_lstar: short write to %s\n", gname.c_str());
    return 2;
  }
  return 1;
}
