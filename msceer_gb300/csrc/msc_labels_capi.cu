// extern "C" entry points of the labeling chain (include/msc_gpu.h): host-side
// orchestration of the K3/K4/K5 kernels for ondemandaccurate's ascending and
// descending 3-manifold labels (ondemandaccurate.cxx:795-948).
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <queue>
#include <string>
#include <vector>

#include "../../include/msc_gpu.h"
#include "label_common.cuh"

namespace msc {
struct IntegParams {
  float ethresh, gthresh;
  int iteration_limit;
  double max_step;
  int step_mult;
};
struct SpreadOrder {
  int nlev;
  int64_t start[48], stride[48], offset[49];
};
cudaError_t launch_integrate_pass1(const float4* G, const VolDims& V, const IntegParams& P, const SpreadOrder& S,
                                   int32_t* lab, int num_sms, cudaStream_t stream);
cudaError_t launch_boundary_set(const int32_t* lab, const uint8_t* state, const VolDims& V, int64_t* list, int* n,
                                uint32_t* queued, int num_sms, cudaStream_t stream);
cudaError_t launch_fixup(const double* G, const VolDims& V, const IntegParams& P, int32_t* lab, uint8_t* state,
                         const int64_t* list, int n, int64_t* next, int* n_next, uint32_t* queued, int num_sms,
                         cudaStream_t stream);
cudaError_t launch_clean(const int32_t* lab, const float* f, const VolDims& V, int dir, int64_t* parent, int64_t* target,
                         int32_t* out, int num_sms, cudaStream_t stream);
cudaError_t launch_central_diff(int nd, int layout, const float* f, void* out, const GradDims& D, int num_sms,
                                cudaStream_t stream);
}  // namespace msc

namespace {

thread_local std::string t_err;

int fail(int code, const std::string& m) {
  t_err = m;
  return code;
}

#define LCUDA(call, what)                                                                              \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess)                                                                             \
      return fail(e_ == cudaErrorMemoryAllocation ? MSC_ERR_OOM : MSC_ERR_CUDA,                       \
                  std::string(what) + ": " + cudaGetErrorString(e_));                                  \
  } while (0)

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 148;
  return n;
}

// Small helper kernels of the orchestration.
__global__ void iota_kernel(int32_t* a, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}
__global__ void fill_i32_kernel(int32_t* a, int64_t n, int32_t v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}
__global__ void terminal_state_kernel(const int32_t* lab, uint8_t* state, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (state[i] != msc::kStSeed) state[i] = lab[i] >= 0 ? msc::kStTerminal : msc::kStUnassigned;
}
// stage snapshot: internal "reached no region" reads as the reference's -1
__global__ void snapshot_kernel(const int32_t* lab, int32_t* out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = lab[i] == msc::kLabelNone ? -1 : lab[i];
}
// SetGradExplicit(seed, 0) (gi_numeric_integrator_path_compressing.h:118-123), both copies
__global__ void zero_seed_grad_kernel(const int64_t* seed, int n, float4* g32, double* g64) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int64_t s = seed[e];
    g32[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    g64[3 * s] = 0.0;
    g64[3 * s + 1] = 0.0;
    g64[3 * s + 2] = 0.0;
  }
}

// UFMergeGraph::SimplifyToThreshold (gi_extrema_region_builder.h:98-145, 232-245) on
// the arcs that can merge at all.
struct HostArc {
  int64_t saddle;
  int32_t e1, e2;
  float sval, pers;
};
struct ArcOrder {  // priority_queue top = smallest persistence, then smallest saddle
  bool operator()(const HostArc& a, const HostArc& b) const {
    if (a.pers > b.pers) return true;
    if (a.pers < b.pers) return false;
    return a.saddle > b.saddle;
  }
};

void host_merge(int dir, float threshold, std::vector<msc::Arc>& arcs, const std::vector<int64_t>& cells,
                const std::vector<int64_t>& hv, const std::vector<float>& fval, std::vector<int32_t>& rep) {
  const int n = (int)cells.size();
  rep.resize(n);
  for (int i = 0; i < n; i++) rep[i] = i;
  auto find = [&](int32_t x) {
    int32_t r = x;
    while (rep[r] != r) r = rep[r];
    while (rep[x] != r) {
      int32_t nx = rep[x];
      rep[x] = r;
      x = nx;
    }
    return r;
  };
  // lessThan of TopologicalMaxVertexMeshFunction (gi_topological_max_vertex_mesh_function.h:47-58)
  auto cell_less = [&](int a, int b) {
    if (fval[a] < fval[b]) return true;
    if (fval[b] < fval[a]) return false;
    if (hv[a] < hv[b]) return true;
    if (hv[b] < hv[a]) return false;
    return cells[a] < cells[b];
  };
  std::priority_queue<HostArc, std::vector<HostArc>, ArcOrder> pq;
  for (auto& a : arcs) pq.push({a.saddle, a.e1, a.e2, a.sval, a.pers});
  const bool min_hier = dir < 0;
  while (!pq.empty()) {
    HostArc m = pq.top();
    pq.pop();
    if (m.pers > threshold) continue;
    const int32_t r1 = find(m.e1), r2 = find(m.e2);
    if (r1 == r2) continue;
    if (m.e1 != r1 || m.e2 != r2) {
      const float d1 = std::fabs(m.sval - fval[r2]);
      const float d2 = std::fabs(m.sval - fval[r1]);
      if (d1 < d2) {
        if (d1 > threshold) continue;
        m.pers = d1;
        m.e1 = r2;
        m.e2 = r1;
      } else {
        if (d2 > threshold) continue;
        m.pers = d2;
        m.e1 = r1;
        m.e2 = r2;
      }
      pq.push(m);
      continue;
    }
    if (cell_less(r1, r2) ^ min_hier) rep[r1] = rep[r2];
    else rep[r2] = rep[r1];
  }
  for (int i = 0; i < n; i++) rep[i] = find(i);
}

// Device scratch of one call, freed in stream order.
struct Pool {
  cudaStream_t st;
  std::vector<void*> ptrs;
  explicit Pool(cudaStream_t s) : st(s) {}
  ~Pool() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
  template <class T>
  cudaError_t get(T** out, size_t count) {
    void* p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, count * sizeof(T) + 16, st);
    if (e == cudaSuccess) {
      ptrs.push_back(p);
      *out = reinterpret_cast<T*>(p);
    }
    return e;
  }
};

int read_int(const int* d, int* h, cudaStream_t st) {
  LCUDA(cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, st), "read counter");
  LCUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  return MSC_OK;
}

int labels_impl(const float* f, const uint8_t* grad, const int64_t* dims, const msc_integ_params* p, int32_t* out_asc,
                int32_t* out_dsc, int32_t* stages, cudaStream_t st) {
  if (!dims || dims[0] < 2 || dims[1] < 2 || dims[2] < 2 || dims[0] > (1 << 20) || dims[1] > (1 << 20) ||
      dims[2] > (1 << 20))
    return fail(MSC_ERR_BAD_DIMS, "labeling needs 2 <= X, Y, Z");
  if (!f || !grad || !p || (!out_asc && !out_dsc)) return fail(MSC_ERR_NULL_POINTER, "null argument");
  msc::VolDims V{dims[0], dims[1], dims[2], 2 * dims[0] - 1, 2 * dims[1] - 1, 2 * dims[2] - 1, 0, 0};
  V.cs1 = V.dX;
  V.cs2 = V.dX * V.dY;
  const int64_t N = V.X * V.Y * V.Z;
  if (N >= ((int64_t)1 << 31)) return fail(MSC_ERR_BAD_DIMS, "labeling supports fewer than 2^31 vertices");
  const int sms = sm_count();
  const int grid = sms * 8;
  Pool pool(st);
  float4* g32;
  double* g64;
  int32_t *lab, *key, *rep, *name;
  uint8_t *state, *tiles;
  int64_t *ext_cells, *saddles, *hv, *seed, *list_a, *list_b, *parent, *target;
  float* fval;
  msc::Arc* arcs;
  uint32_t* queued;
  int* counters;  // [0] n_ext [1] n_sad [2] n_arcs [3] changed [4] err [5] n_list [6] n_next
  const int64_t ntiles = msc::terminal_num_tiles(V);
  LCUDA(pool.get(&g32, N), "alloc");
  LCUDA(pool.get(&g64, 3 * N), "alloc");
  LCUDA(pool.get(&lab, N), "alloc");
  LCUDA(pool.get(&key, N), "alloc");
  LCUDA(pool.get(&state, N), "alloc");
  LCUDA(pool.get(&ext_cells, N), "alloc");
  LCUDA(pool.get(&saddles, 3 * N), "alloc");
  LCUDA(pool.get(&list_a, N), "alloc");
  LCUDA(pool.get(&list_b, N), "alloc");
  LCUDA(pool.get(&queued, N / 32 + 1), "alloc");
  LCUDA(pool.get(&tiles, 2 * ntiles), "alloc");
  LCUDA(pool.get(&counters, 8), "alloc");
  msc::GradDims GD{};
  for (int a = 0; a < 3; a++) {
    GD.v[a] = dims[a];
    GD.d[a] = 2 * dims[a] - 1;
  }
  LCUDA(msc::launch_central_diff(3, 1, f, g32, GD, sms, st), "gradient f32");
  LCUDA(msc::launch_central_diff(3, 2, f, g64, GD, sms, st), "gradient f64");

  for (int pass = 0; pass < 2; pass++) {
    int32_t* out = pass == 0 ? out_asc : out_dsc;
    if (!out) continue;
    const int dir = pass == 0 ? -1 : 1;
    LCUDA(cudaMemsetAsync(counters, 0, 8 * sizeof(int), st), "memset");
    fill_i32_kernel<<<grid, 256, 0, st>>>(key, N, -1);
    LCUDA(msc::launch_find_critical(grad, V, dir, key, ext_cells, counters, saddles, counters + 1, sms, st), "critical");
    int h[8];
    LCUDA(cudaMemcpyAsync(h, counters, 2 * sizeof(int), cudaMemcpyDeviceToHost, st), "read");
    LCUDA(cudaStreamSynchronize(st), "sync");
    const int n_ext = h[0], n_sad = h[1];
    LCUDA(pool.get(&hv, n_ext + 1), "alloc");
    LCUDA(pool.get(&fval, n_ext + 1), "alloc");
    LCUDA(pool.get(&seed, n_ext + 1), "alloc");
    LCUDA(pool.get(&rep, n_ext + 1), "alloc");
    LCUDA(pool.get(&name, n_ext + 1), "alloc");
    LCUDA(pool.get(&arcs, n_sad + 1), "alloc");
    LCUDA(msc::launch_extremum_info(f, V, dir, ext_cells, n_ext, hv, fval, seed, sms, st), "extremum info");
    LCUDA(msc::launch_trace_arcs(grad, f, V, dir, saddles, n_sad, key, p->presimp_threshold, arcs, counters + 2,
                                 counters + 4, sms, st),
          "trace arcs");
    int n_arcs = 0;
    if (int rc = read_int(counters + 2, &n_arcs, st)) return rc;
    if (n_ext > 0) iota_kernel<<<(n_ext + 255) / 256, 256, 0, st>>>(rep, n_ext);
    if (n_arcs > 0) {
      // the few arcs that can merge: exact priority-queue simplification on the host
      std::vector<msc::Arc> ha(n_arcs);
      std::vector<int64_t> hcells(n_ext), hhv(n_ext);
      std::vector<float> hf(n_ext);
      LCUDA(cudaMemcpyAsync(ha.data(), arcs, n_arcs * sizeof(msc::Arc), cudaMemcpyDeviceToHost, st), "read arcs");
      LCUDA(cudaMemcpyAsync(hcells.data(), ext_cells, n_ext * sizeof(int64_t), cudaMemcpyDeviceToHost, st), "read");
      LCUDA(cudaMemcpyAsync(hhv.data(), hv, n_ext * sizeof(int64_t), cudaMemcpyDeviceToHost, st), "read");
      LCUDA(cudaMemcpyAsync(hf.data(), fval, n_ext * sizeof(float), cudaMemcpyDeviceToHost, st), "read");
      LCUDA(cudaStreamSynchronize(st), "sync");
      std::vector<int32_t> hrep;
      host_merge(dir, p->presimp_threshold, ha, hcells, hhv, hf, hrep);
      LCUDA(cudaMemcpyAsync(rep, hrep.data(), n_ext * sizeof(int32_t), cudaMemcpyHostToDevice, st), "write rep");
      LCUDA(cudaStreamSynchronize(st), "sync");
    }
    fill_i32_kernel<<<grid, 256, 0, st>>>(lab, N, -1);
    fill_i32_kernel<<<(n_ext + 256) / 256, 256, 0, st>>>(name, n_ext + 1, INT_MAX);
    LCUDA(cudaMemsetAsync(state, 0, (size_t)N, st), "memset");
    LCUDA(msc::launch_group_seeds(rep, seed, n_ext, name, lab, state, sms, st), "seeds");

    // certain terminal regions: tile passes to the fixpoint
    const uint8_t* din = nullptr;
    uint8_t* dout = tiles;
    for (int64_t passes = 0;; passes++) {
      LCUDA(cudaMemsetAsync(counters + 3, 0, sizeof(int), st), "memset");
      LCUDA(cudaMemsetAsync(dout, 0, (size_t)ntiles, st), "memset");
      LCUDA(msc::launch_terminal_pass(f, lab, V, dir, din, dout, counters + 3, counters + 4, sms, st), "regions");
      int changed = 0;
      if (int rc = read_int(counters + 3, &changed, st)) return rc;
      if (!changed) break;
      if (passes > ntiles + 2) return fail(MSC_ERR_ITER_LIMIT, "terminal regions did not converge");
      din = dout;
      dout = (dout == tiles) ? tiles + ntiles : tiles;
    }
    if (stages) snapshot_kernel<<<grid, 256, 0, st>>>(lab, stages + (2 * pass) * N, N);
    terminal_state_kernel<<<grid, 256, 0, st>>>(lab, state, N);
    if (n_ext > 0) zero_seed_grad_kernel<<<(n_ext + 255) / 256, 256, 0, st>>>(seed, n_ext, g32, g64);

    // first pass with path compression, in the reference's spread order
    msc::IntegParams P{p->error_threshold, p->gradient_threshold, p->iteration_limit, (double)p->max_step, dir};
    msc::SpreadOrder S{};
    S.nlev = 0;
    S.offset[0] = 0;
    for (int64_t kk = 1; kk <= N * 4 && S.nlev < 48; kk *= 2) {
      const int64_t start = N / kk, stride = (N * 2) / kk;
      if (stride == 0 || start >= N) continue;
      S.start[S.nlev] = start;
      S.stride[S.nlev] = stride;
      S.offset[S.nlev + 1] = S.offset[S.nlev] + (N - start + stride - 1) / stride;
      S.nlev++;
    }
    LCUDA(msc::launch_integrate_pass1(g32, V, P, S, lab, sms, st), "integrate");

    // fix-up waves (FP64) until no label changes reopen a neighbour
    LCUDA(cudaMemsetAsync(queued, 0, (N / 32 + 1) * sizeof(uint32_t), st), "memset");
    LCUDA(cudaMemsetAsync(counters + 5, 0, 2 * sizeof(int), st), "memset");
    LCUDA(msc::launch_boundary_set(lab, state, V, list_a, counters + 5, queued, sms, st), "boundary set");
    int n_list = 0;
    if (int rc = read_int(counters + 5, &n_list, st)) return rc;
    int64_t* cur = list_a;
    int64_t* nxt = list_b;
    for (int64_t waves = 0; n_list > 0; waves++) {
      if (waves > N) return fail(MSC_ERR_ITER_LIMIT, "fix-up did not converge");
      LCUDA(cudaMemsetAsync(counters + 6, 0, sizeof(int), st), "memset");
      LCUDA(msc::launch_fixup(g64, V, P, lab, state, cur, n_list, nxt, counters + 6, queued, sms, st), "fix-up");
      if (int rc = read_int(counters + 6, &n_list, st)) return rc;
      int64_t* t = cur;
      cur = nxt;
      nxt = t;
    }
    if (stages) snapshot_kernel<<<grid, 256, 0, st>>>(lab, stages + (2 * pass + 1) * N, N);

    // isolated-region cleaner
    LCUDA(pool.get(&parent, N), "alloc");
    LCUDA(pool.get(&target, N), "alloc");
    LCUDA(msc::launch_clean(lab, f, V, dir, parent, target, out, sms, st), "clean");
  }
  int err = 0;
  if (int rc = read_int(counters + 4, &err, st)) return rc;
  if (err & msc::kErrLocalQueue) return fail(MSC_ERR_QUEUE_OVERFLOW, "tile queue overflow");
  if (err & msc::kErrIterLimit) return fail(MSC_ERR_ITER_LIMIT, "V-path walk exceeded its bound (invalid gradient?)");
  return MSC_OK;
}

}  // namespace

extern "C" {

const char* msc_labels_last_error_string(void) { return t_err.c_str(); }

int msc_integrated_labels_3d(const float* f, const uint8_t* grad, const int64_t dims[3], const msc_integ_params* params,
                             int32_t* labels_asc, int32_t* labels_dsc, msc_stream_t stream) {
  return labels_impl(f, grad, dims, params, labels_asc, labels_dsc, nullptr, (cudaStream_t)stream);
}

int msc_integrated_labels_3d_stages(const float* f, const uint8_t* grad, const int64_t dims[3],
                                    const msc_integ_params* params, int32_t* labels_asc, int32_t* labels_dsc,
                                    int32_t* stages, msc_stream_t stream) {
  return labels_impl(f, grad, dims, params, labels_asc, labels_dsc, stages, (cudaStream_t)stream);
}

}  // extern "C"
