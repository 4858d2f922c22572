// ondemandaccurate -- drop-in for MSCEER's ondemandaccurate/ondemandaccurate.cxx (its
// accurate 3-manifold mode) on one GB300.
//
// Same command line (ondemandaccurate.cxx:158-185):
//     ondemandaccurate X Y Z filename error_threshold grad_threshold maxnumiter
//                      needASC1 needDSC1 needASC2 needDSC2 PresimpThresh
//                      [parallelism] [outputdebug]
// reads X*Y*Z float32 (x fastest) from `filename` and writes `filename.grad`:
//   * nothing accurate requested: the lower-star .grad (:770-775);
//   * needASC2 / needDSC2: the .grad made conforming to the integrated ascending /
//     descending 3-manifolds (:795-1063): extremum graph and terminal regions,
//     path-compressing streamline integration with the adaptive Euler advector, the
//     isolated-region cleaner, the restriction labels of the region boundaries and the
//     re-pairing of the touched lower stars.
// plus the timing file `filename.NNN.gtime.txt` (:721-723; NNN the parallelism) with
// "task start end duration" lines in milliseconds.  With outputdebug the ascending
// labels are dumped as int32 per vertex, as :832-852 does: extremal_asc.raw (terminal
// regions), newintegrator_asc.raw (integrated), newintegrator_cleaned_asc.raw
// (cleaned), and boundaries_<dX>x<dY>x<dZ>.raw (one restriction byte per cell, :1005-1011).
// Labels name each region by the smallest seed vertex of its extremum (the reference
// numbers regions in hash-map order, which changes from run to run).
//
// The integration step bound is the reference's compile-time MAX_STEP_IN_GRID_CELLS
// (gi_adaptive_euler_advector.h:12, 0.5 voxel); the environment variable
// MSC_MAX_STEP_IN_GRID_CELLS sets it as that define does.  parallelism is accepted and
// ignored (the work runs on the GPU).  The saddle-line modes (needASC1 / needDSC1,
// :1068 on) are not provided: the program says so and exits with status 2.  Exit
// status otherwise as the reference: 1 after a completed run, 0 after the usage
// message (also printed, instead of reading past argv, when fewer than the 12
// positional arguments are given); a failure prints the library error and returns 2.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "msc_gpu.h"

namespace {

struct Timing {
  FILE* f = nullptr;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now(), task;
  void start() { task = std::chrono::steady_clock::now(); }
  void end(const char* what) {
    const auto now = std::chrono::steady_clock::now();
    auto ms = [&](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
      return (long long)std::chrono::duration_cast<std::chrono::milliseconds>(b - a).count();
    };
    if (f) fprintf(f, "%s %lld %lld %lld\n", what, ms(t0, task), ms(t0, now), ms(task, now));
    printf("TIMING: %s %lld %lld %lld\n", what, ms(t0, task), ms(t0, now), ms(task, now));
  }
  ~Timing() {
    if (f) fclose(f);
  }
};

int fail_lib(const char* what, int rc) {
  fprintf(stderr, "ondemandaccurate: %s: %s (status %d)\n", what,
          std::string(msc_last_error_string()).empty() ? msc_labels_last_error_string() : msc_last_error_string(), rc);
  return 2;
}

int fail_cuda(const char* what, cudaError_t e) {
  fprintf(stderr, "ondemandaccurate: %s: %s\n", what, cudaGetErrorString(e));
  return 2;
}

bool write_file(const std::string& name, const void* data, size_t bytes) {
  FILE* fo = fopen(name.c_str(), "wb");
  if (!fo) return false;
  const size_t put = fwrite(data, 1, bytes, fo);
  fclose(fo);
  return put == bytes;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 13) {
    printf("Usage: X Y Z filename error_threshold grad_threshold maxnumiter needASC1 needDSC1 needASC2 needDSC2 "
           "PresimpThesh [parallelism=ompmaxnumthreads] [outputdebug=0] [integrationinteraltimer=0]\n");
    return 0;
  }
  int X = 0, Y = 0, Z = 0, iteration_limit = 0, need_asc1 = 0, need_dsc1 = 0, need_asc3 = 0, need_dsc3 = 0;
  int parallelism = -1, output_debug = 0;
  float error_threshold = 0.f, gradient_threshold = 0.f, presimp = 0.f;
  sscanf(argv[1], "%d", &X);
  sscanf(argv[2], "%d", &Y);
  sscanf(argv[3], "%d", &Z);
  const std::string filename(argv[4]);
  sscanf(argv[5], "%f", &error_threshold);
  sscanf(argv[6], "%f", &gradient_threshold);
  sscanf(argv[7], "%d", &iteration_limit);
  sscanf(argv[8], "%d", &need_asc1);
  sscanf(argv[9], "%d", &need_dsc1);
  sscanf(argv[10], "%d", &need_asc3);
  sscanf(argv[11], "%d", &need_dsc3);
  sscanf(argv[12], "%f", &presimp);
  if (argc >= 14) sscanf(argv[13], "%d", &parallelism);
  if (argc >= 15) sscanf(argv[14], "%d", &output_debug);
  printf("dims=(%d,%d,%d)\nfile=%s\nintegration parameters: e=%f, gt=%f, il=%d\n"
         "ondemandacc: a1=%d, d1=%d, a2=%d, d2=%d, ps=%f\npar=%d\n",
         X, Y, Z, argv[4], error_threshold, gradient_threshold, iteration_limit, need_asc1, need_dsc1, need_asc3,
         need_dsc3, presimp, parallelism);
  if (need_asc1 || need_dsc1) {
    fprintf(stderr, "ondemandaccurate: the saddle-line modes (needASC1 / needDSC1) are not provided\n");
    return 2;
  }
  float max_step = 0.5f;
  if (const char* e = std::getenv("MSC_MAX_STEP_IN_GRID_CELLS")) max_step = (float)atof(e);

  const int64_t dims[3] = {X, Y, Z};
  const int64_t ncells = msc_num_cells_3d(dims);
  if (ncells < 0 || X < 2 || Y < 2 || Z < 2) {
    fprintf(stderr, "ondemandaccurate: invalid dimensions %d %d %d\n", X, Y, Z);
    return 2;
  }
  const size_t nv = (size_t)X * (size_t)Y * (size_t)Z;
  std::vector<float> f(nv);
  FILE* fin = fopen(filename.c_str(), "rb");
  if (!fin) {
    fprintf(stderr, "ondemandaccurate: cannot open %s\n", filename.c_str());
    return 2;
  }
  const size_t got = fread(f.data(), sizeof(float), nv, fin);
  fclose(fin);
  if (got != nv) {
    fprintf(stderr, "ondemandaccurate: %s holds %zu of %zu values\n", filename.c_str(), got, nv);
    return 2;
  }

  Timing tm;
  char tname[2048];
  snprintf(tname, sizeof(tname), "%s.%03d.gtime.txt", filename.c_str(), parallelism);
  tm.f = fopen(tname, "w");

  float* df = nullptr;
  uint8_t* dg = nullptr;
  int32_t *dasc = nullptr, *ddsc = nullptr, *dstages = nullptr;
  uint8_t* drl = nullptr;
  struct Free {
    std::vector<void*> p;
    ~Free() {
      for (void* q : p) cudaFree(q);
    }
  } fr;
  cudaError_t e;
  if ((e = cudaMalloc(&df, nv * sizeof(float))) != cudaSuccess) return fail_cuda("cudaMalloc", e);
  fr.p.push_back(df);
  if ((e = cudaMalloc(&dg, (size_t)ncells)) != cudaSuccess) return fail_cuda("cudaMalloc", e);
  fr.p.push_back(dg);
  if ((e = cudaMemcpy(df, f.data(), nv * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail_cuda("cudaMemcpy", e);

  tm.start();
  if (int rc = msc_lower_star_grad_3d(df, dims, dg, nullptr)) return fail_lib("lower-star gradient", rc);
  cudaDeviceSynchronize();
  tm.end("Topological Robins0");

  if (need_asc3 || need_dsc3) {
    if (need_asc3) {
      if ((e = cudaMalloc(&dasc, nv * sizeof(int32_t))) != cudaSuccess) return fail_cuda("cudaMalloc", e);
      fr.p.push_back(dasc);
    }
    if (need_dsc3) {
      if ((e = cudaMalloc(&ddsc, nv * sizeof(int32_t))) != cudaSuccess) return fail_cuda("cudaMalloc", e);
      fr.p.push_back(ddsc);
    }
    if (output_debug) {
      if ((e = cudaMalloc(&dstages, 4 * nv * sizeof(int32_t))) != cudaSuccess) return fail_cuda("cudaMalloc", e);
      fr.p.push_back(dstages);
      if ((e = cudaMalloc(&drl, (size_t)ncells)) != cudaSuccess) return fail_cuda("cudaMalloc", e);
      fr.p.push_back(drl);
    }
    msc_integ_params p{};
    p.error_threshold = error_threshold;
    p.gradient_threshold = gradient_threshold;
    p.iteration_limit = iteration_limit;
    p.max_step = max_step;
    p.presimp_threshold = presimp;
    p.precision = 0;
    tm.start();
    const int rc = dstages ? msc_integrated_labels_3d_stages(df, dg, dims, &p, dasc, ddsc, dstages, nullptr)
                           : msc_integrated_labels_3d(df, dg, dims, &p, dasc, ddsc, nullptr);
    if (rc) return fail_lib("integrated labels", rc);
    tm.end("NumericalTracing Labels");
    tm.start();
    int64_t touched = 0;
    if (int rc2 = msc_conforming_grad_3d(df, dasc, ddsc, dims, dg, drl, &touched, nullptr))
      return fail_lib("conforming gradient", rc2);
    printf("re-paired %lld vertices\n", (long long)touched);
    tm.end("Topological ConformingGrad");
    if (output_debug && dasc) {
      std::vector<int32_t> h(nv);
      const struct {
        const int32_t* src;
        const char* name;
      } dumps[3] = {{dstages, "extremal_asc.raw"}, {dstages + nv, "newintegrator_asc.raw"},
                    {dasc, "newintegrator_cleaned_asc.raw"}};
      for (const auto& d : dumps) {
        if ((e = cudaMemcpy(h.data(), d.src, nv * sizeof(int32_t), cudaMemcpyDeviceToHost)) != cudaSuccess)
          return fail_cuda("cudaMemcpy", e);
        printf("writing file %s\n", d.name);
        if (!write_file(d.name, h.data(), nv * sizeof(int32_t))) {
          fprintf(stderr, "ondemandaccurate: cannot write %s\n", d.name);
          return 2;
        }
      }
    }
    if (output_debug) {
      std::vector<uint8_t> h((size_t)ncells);
      if ((e = cudaMemcpy(h.data(), drl, (size_t)ncells, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return fail_cuda("cudaMemcpy", e);
      char name[256];
      snprintf(name, sizeof(name), "boundaries_%dx%dx%d.raw", 2 * X - 1, 2 * Y - 1, 2 * Z - 1);
      if (!write_file(name, h.data(), h.size())) {
        fprintf(stderr, "ondemandaccurate: cannot write %s\n", name);
        return 2;
      }
    }
  } else {
    printf("no accuraccy needed, outputting\n");
  }

  std::vector<uint8_t> grad((size_t)ncells);
  if ((e = cudaMemcpy(grad.data(), dg, (size_t)ncells, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return fail_cuda("cudaMemcpy", e);
  const std::string gname = filename + ".grad";
  printf("outputting to file %s\n", gname.c_str());
  if (!write_file(gname, grad.data(), grad.size())) {
    fprintf(stderr, "ondemandaccurate: cannot write %s\n", gname.c_str());
    return 2;
  }
  return 1;
}
