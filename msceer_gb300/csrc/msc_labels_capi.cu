// extern "C" entry points of the labeling chain (include/msc_gpu.h): host-side
// orchestration of the K3/K4/K5 kernels for ondemandaccurate's ascending and
// descending 3-manifold labels (ondemandaccurate.cxx:795-948).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <functional>
#include <map>
#include <mutex>
#include <queue>
#include <thread>
#include <string>
#include <utility>
#include <vector>

#include "../../include/msc_gpu.h"
#include "../../include/msc_triage.h"
#include "label_common.cuh"
#include "triage.cuh"


namespace {

thread_local std::string t_err;
// per direction (asc, dsc): fix-up re-decisions, of which in FP64
thread_local int64_t t_stats[4];
thread_local int64_t t_trips[6];

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

// Phase trace (MSC_LABELS_TRACE=1): a timing event per phase boundary of each
// direction, printed to stderr at the end of the call -- device time of each boundary
// and host time of its enqueue, both from the call's first mark.
struct TraceMark {
  int dir;
  std::string what;
  cudaEvent_t ev;
  std::chrono::steady_clock::time_point host;
};
std::mutex g_trace_mu;
std::vector<TraceMark> g_trace;
bool trace_on() {
  static const bool on = [] {
    const char* e = std::getenv("MSC_LABELS_TRACE");
    return e && *e && *e != '0';
  }();
  return on;
}
void trace_mark(cudaStream_t st, int dir, const std::string& what) {
  if (!trace_on()) return;
  TraceMark m{dir, what, nullptr, std::chrono::steady_clock::now()};
  if (cudaEventCreate(&m.ev) != cudaSuccess) return;
  cudaEventRecord(m.ev, st);
  std::lock_guard<std::mutex> lk(g_trace_mu);
  g_trace.push_back(m);
}
void trace_dump() {
  if (!trace_on()) return;
  std::lock_guard<std::mutex> lk(g_trace_mu);
  if (g_trace.empty()) return;
  const cudaEvent_t e0 = g_trace.front().ev;
  const auto h0 = g_trace.front().host;
  for (const TraceMark& m : g_trace) {
    float ms = -1.f;
    cudaEventSynchronize(m.ev);
    cudaEventElapsedTime(&ms, e0, m.ev);
    const double hms = std::chrono::duration<double, std::milli>(m.host - h0).count();
    std::fprintf(stderr, "[labels] %s %-24s device %9.3f ms  host %9.3f ms\n", m.dir < 0 ? "asc" : "dsc",
                 m.what.c_str(), ms, hms);
  }
  // the first mark's event is every line's base: destroy the events only now
  for (const TraceMark& m : g_trace) cudaEventDestroy(m.ev);
  g_trace.clear();
}

}  // namespace

void msc::label_trace(cudaStream_t st, int dir, const char* what) { trace_mark(st, dir, what); }

namespace {

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
// caller labels into the internal form: the reference's -1 ("none") reads as kLabelNone
__global__ void none_in_kernel(const int32_t* in, int32_t* lab, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    lab[i] = in[i] == -1 ? msc::kLabelNone : in[i];
}
// stage snapshot: internal "reached no region" reads as the reference's -1
__global__ void snapshot_kernel(const int32_t* lab, int32_t* out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = lab[i] == msc::kLabelNone ? -1 : lab[i];
}
// the extrema that the mergeable arcs touch, gathered for the host merge
// the host merge's changed representatives: rep[pairs[2k]] = pairs[2k + 1]
__global__ void scatter_rep_kernel(const int32_t* pairs, int m, int32_t* rep) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) rep[pairs[2 * i]] = pairs[2 * i + 1];
}
// SetGradExplicit(seed, 0) (gi_numeric_integrator_path_compressing.h:118-123): the FP32
// gradient, and the bit that makes the FP64 advector's corner gradient zero
__global__ void zero_seed_grad_kernel(const int64_t* seed, int n, float4* g32, uint32_t* zeroed) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int64_t s = seed[e];
    g32[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    atomicOr(&zeroed[s >> 5], 1u << (s & 31));
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

// Device scratch of one call, freed in stream order into the scratch pool.
struct Pool {
  cudaStream_t st;
  cudaMemPool_t mp = nullptr;
  cudaError_t init_err;
  std::vector<void*> ptrs;
  explicit Pool(cudaStream_t s) : st(s) { init_err = msc::scratch_pool(&mp); }
  ~Pool() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
  template <class T>
  cudaError_t get(T** out, size_t count) {
    if (init_err != cudaSuccess) return init_err;
    void* p = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&p, count * sizeof(T) + 16, mp, st);
    if (e == cudaSuccess) {
      ptrs.push_back(p);
      *out = reinterpret_cast<T*>(p);
    }
    return e;
  }
};

// Pinned host words for the counter reads that steer the host loop.  A copy into
// pageable memory held up the other direction's host thread in its CUDA calls until the
// copy (and so the kernel before it) had finished; a pinned one does not.  The buffers
// are reused across calls and never freed (freeing pinned memory synchronises).
constexpr size_t kPinnedBytes = 256;
std::mutex g_pin_mu;
std::vector<void*> g_pin_free;
void* pinned_get() {
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    if (!g_pin_free.empty()) {
      void* p = g_pin_free.back();
      g_pin_free.pop_back();
      return p;
    }
  }
  void* p = nullptr;
  return cudaMallocHost(&p, kPinnedBytes) == cudaSuccess ? p : nullptr;
}
void pinned_put(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_pin_free.push_back(p);
}

// Shared state of one labeling call.
struct LabelCtx {
  cudaStream_t st;
  Pool pool;
  int sms = 0, grid = 0;
  msc::VolDims V{};
  int64_t N = 0, ntiles = 0;
  const float* f = nullptr;
  const uint8_t* grad = nullptr;
  const msc_integ_params* p = nullptr;
  float4* g32 = nullptr;
  uint32_t* zeroed = nullptr;  // a bit per vertex whose gradient is zeroed (the FP64 advector's)
  int32_t* key = nullptr;
  int64_t *ext_cells = nullptr, *saddles = nullptr, *list_a = nullptr, *list_b = nullptr, *amb = nullptr;
  int64_t* list_c = nullptr;  // a fix-up wave's members without a streamline end yet
  uint32_t* queued = nullptr;
  uint8_t* tiles = nullptr;
  int* counters = nullptr;  // [0] n_ext [1] n_sad [2] n_arcs [3] changed [4] err [5] n_list / wave members
                            // without an end [6] n_next [7] n_amb [8, 10) cleaner [10] long chain
                            // [12] vertices whose ends are computed ahead of the waves
                            // [13], [14] terminal-walk frontier lengths
  unsigned long long* work = nullptr;  // [0] claimed fix-up items, [48, 51) advection iterations (first
                                       // pass, FP32, FP64), [56] FP64 claims
  void* hpin = nullptr;                // kPinnedBytes of pinned host memory (pinned_get)
  // the streamline ends computed ahead of the fix-up waves, beside the first pass
  cudaStream_t ends_st = nullptr;
  cudaEvent_t ends_go = nullptr, ends_done = nullptr;
  explicit LabelCtx(cudaStream_t s) : st(s), pool(s) {}
  ~LabelCtx() {
    if (ends_st) cudaStreamSynchronize(ends_st);
    cudaStreamSynchronize(st);  // no copy into hpin in flight
    pinned_put(hpin);
    if (ends_go) cudaEventDestroy(ends_go);
    if (ends_done) cudaEventDestroy(ends_done);
    if (ends_st) cudaStreamDestroy(ends_st);
  }
  LabelCtx(const LabelCtx&) = delete;
  LabelCtx& operator=(const LabelCtx&) = delete;
};

// n values of device memory, read through the context's pinned words
template <class T>
int read_dev(LabelCtx& c, const T* d, int n, T* out) {
  static_assert(sizeof(T) <= 8, "counters");
  if ((size_t)n * sizeof(T) > kPinnedBytes) return fail(MSC_ERR_CUDA, "counter read too large");
  LCUDA(cudaMemcpyAsync(c.hpin, d, n * sizeof(T), cudaMemcpyDeviceToHost, c.st), "read counters");
  LCUDA(cudaStreamSynchronize(c.st), "cudaStreamSynchronize");
  std::memcpy(out, c.hpin, n * sizeof(T));
  return MSC_OK;
}

// One direction's labels between the phases.
struct DirLabels {
  int dir = -1;
  std::function<int()> on_seeds;         // called once the seed list is on the stream (prepare_direction)
  std::function<int()> before_integration;  // called at the end of prepare_direction
  int64_t trips[3] = {0, 0, 0};  // advection iterations: first pass, FP32 fix-up, FP64 re-decisions
  int32_t* lab = nullptr;
  uint8_t* state = nullptr;
  int64_t* seed = nullptr;
  int n_ext = 0;
  bool seeds_zeroed = false;  // the gradient at this direction's seeds is zero on the stream
  bool trips_zeroed = false;  // the iteration counters (work[48, 51)) are zero on the stream
};

int setup_ctx(LabelCtx& c, const float* f, const uint8_t* grad, const int64_t* dims, const msc_integ_params* p) {
  if (!dims || dims[0] < 2 || dims[1] < 2 || dims[2] < 2 || dims[0] > (1 << 20) || dims[1] > (1 << 20) ||
      dims[2] > (1 << 20))
    return fail(MSC_ERR_BAD_DIMS, "labeling needs 2 <= X, Y, Z");
  if (!f || !grad || !p) return fail(MSC_ERR_NULL_POINTER, "null argument");
  c.V = msc::VolDims{dims[0], dims[1], dims[2], 2 * dims[0] - 1, 2 * dims[1] - 1, 2 * dims[2] - 1, 0, 0};
  c.V.cs1 = c.V.dX;
  c.V.cs2 = c.V.dX * c.V.dY;
  c.N = c.V.X * c.V.Y * c.V.Z;
  if (c.N >= ((int64_t)1 << 31)) return fail(MSC_ERR_BAD_DIMS, "labeling supports fewer than 2^31 vertices");
  c.f = f;
  c.grad = grad;
  c.p = p;
  if (!c.hpin && !(c.hpin = pinned_get())) return fail(MSC_ERR_OOM, "pinned host words");
  c.sms = sm_count();
  c.grid = c.sms * 8;
  c.ntiles = msc::terminal_num_tiles(c.V);
  const int64_t N = c.N;
  LCUDA(c.pool.get(&c.g32, N), "alloc");
  LCUDA(c.pool.get(&c.zeroed, N / 32 + 1), "alloc");
  LCUDA(c.pool.get(&c.key, N), "alloc");
  LCUDA(c.pool.get(&c.ext_cells, N), "alloc");
  LCUDA(c.pool.get(&c.saddles, 3 * N), "alloc");
  LCUDA(c.pool.get(&c.list_a, N), "alloc");
  LCUDA(c.pool.get(&c.list_b, N), "alloc");
  LCUDA(c.pool.get(&c.amb, N), "alloc");
  LCUDA(c.pool.get(&c.list_c, N), "alloc");
  LCUDA(c.pool.get(&c.queued, N / 32 + 1), "alloc");
  LCUDA(c.pool.get(&c.tiles, 2 * c.ntiles), "alloc");
  LCUDA(c.pool.get(&c.counters, 16), "alloc");
  LCUDA(c.pool.get(&c.work, 64), "alloc");
  LCUDA(cudaMemsetAsync(c.counters, 0, 16 * sizeof(int), c.st), "memset");
  msc::GradDims GD{};
  for (int a = 0; a < 3; a++) {
    GD.v[a] = dims[a];
    GD.d[a] = 2 * dims[a] - 1;
  }
  LCUDA(msc::launch_central_diff(3, 1, f, c.g32, GD, c.sms, c.st), "gradient f32");
  LCUDA(cudaMemsetAsync(c.zeroed, 0, (size_t)(N / 32 + 1) * sizeof(uint32_t), c.st), "memset");
  return MSC_OK;
}

// Extremum graph, merge, seeds and certain terminal regions of one direction; leaves
// d.lab (terminal labels, -1 elsewhere) and d.state.
bool terminal_tiles_on() {
  static const bool on = [] {
    const char* e = std::getenv("MSC_TERMINAL_TILES");
    return e && std::atoi(e) == 1;
  }();
  return on;
}

int prepare_direction(LabelCtx& c, DirLabels& d, int32_t* stage_terminal) {
  const int64_t N = c.N;
  const msc::VolDims& V = c.V;
  cudaStream_t st = c.st;
  const int dir = d.dir;
  int32_t *rep, *name;
  int64_t* hv;
  float* fval;
  msc::Arc* arcs;
  LCUDA(c.pool.get(&d.lab, N), "alloc");
  LCUDA(c.pool.get(&d.state, N), "alloc");
  LCUDA(cudaMemsetAsync(c.counters, 0, 3 * sizeof(int), st), "memset");
  ::msc::count_launch();
  fill_i32_kernel<<<c.grid, 256, 0, st>>>(c.key, N, -1);
  LCUDA(msc::launch_find_critical(c.grad, V, dir, c.key, c.ext_cells, c.counters, c.saddles, c.counters + 1, c.sms, st),
        "critical");
  int h[2];
  if (int rc = read_dev(c, c.counters, 2, h)) return rc;
  const int n_ext = h[0], n_sad = h[1];
  d.n_ext = n_ext;
  trace_mark(st, dir, "critical cells");
  LCUDA(c.pool.get(&hv, n_ext + 1), "alloc");
  LCUDA(c.pool.get(&fval, n_ext + 1), "alloc");
  LCUDA(c.pool.get(&d.seed, n_ext + 1), "alloc");
  LCUDA(c.pool.get(&rep, n_ext + 1), "alloc");
  LCUDA(c.pool.get(&name, n_ext + 1), "alloc");
  LCUDA(c.pool.get(&arcs, n_sad + 1), "alloc");
  LCUDA(msc::launch_extremum_info(c.f, V, dir, c.ext_cells, n_ext, hv, fval, d.seed, c.sms, st), "extremum info");
  // the seed list is final here (the merge below changes representatives, not seeds)
  if (d.on_seeds)
    if (int rc = d.on_seeds()) return rc;
  LCUDA(msc::launch_trace_arcs(c.grad, c.f, V, dir, c.saddles, n_sad, c.key, c.p->presimp_threshold, arcs,
                               c.counters + 2, c.counters + 4, c.sms, st),
        "trace arcs");
  int n_arcs = 0;
  if (int rc = read_dev(c, c.counters + 2, 1, &n_arcs)) return rc;
  trace_mark(st, dir, "arcs");
  if (n_ext > 0) {
    ::msc::count_launch();
    iota_kernel<<<(n_ext + 255) / 256, 256, 0, st>>>(rep, n_ext);
  }
  if (n_arcs > 0) {
    // the few arcs that can merge: exact priority-queue simplification on the host, over
    // the extrema those arcs touch (the merge reads no other; a merge over all n_ext
    // extrema copied ~10 M of them at 512^3 for a few hundred arcs)
    std::vector<msc::Arc> ha(n_arcs);
    LCUDA(cudaMemcpyAsync(ha.data(), arcs, n_arcs * sizeof(msc::Arc), cudaMemcpyDeviceToHost, st), "read arcs");
    LCUDA(cudaStreamSynchronize(st), "sync");
    std::vector<int32_t> ids;
    ids.reserve(2 * (size_t)n_arcs);
    for (const msc::Arc& a : ha) {
      if (a.e1 < 0 || a.e1 >= n_ext || a.e2 < 0 || a.e2 >= n_ext)
        return fail(MSC_ERR_CUDA, "arc endpoint outside the extremum list");
      ids.push_back(a.e1);
      ids.push_back(a.e2);
    }
    std::sort(ids.begin(), ids.end());
    ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
    const int m = (int)ids.size();
    // the arcs carry their extrema's cells, highest vertices and values: no gather and
    // no second wait for the GPU (whose SMs the other direction's launches may hold)
    std::vector<int64_t> hcells(m), hhv(m);
    std::vector<float> hf(m);
    for (msc::Arc& a : ha) {
      a.e1 = (int32_t)(std::lower_bound(ids.begin(), ids.end(), a.e1) - ids.begin());
      a.e2 = (int32_t)(std::lower_bound(ids.begin(), ids.end(), a.e2) - ids.begin());
      hcells[a.e1] = a.c1;
      hhv[a.e1] = a.h1;
      hf[a.e1] = a.f1;
      hcells[a.e2] = a.c2;
      hhv[a.e2] = a.h2;
      hf[a.e2] = a.f2;
    }
    std::vector<int32_t> hrep;
    host_merge(dir, c.p->presimp_threshold, ha, hcells, hhv, hf, hrep);
    std::vector<int32_t> pairs;
    for (int i = 0; i < m; i++)
      if (hrep[i] != i) {
        pairs.push_back(ids[i]);
        pairs.push_back(ids[hrep[i]]);
      }
    const int np = (int)pairs.size() / 2;
    if (np > 0) {
      int32_t* dpairs;
      LCUDA(c.pool.get(&dpairs, 2 * (size_t)np), "alloc");
      // (from pageable memory the copy has taken the data when the call returns)
      LCUDA(cudaMemcpyAsync(dpairs, pairs.data(), 2 * np * sizeof(int32_t), cudaMemcpyHostToDevice, st), "write rep");
      ::msc::count_launch();
      scatter_rep_kernel<<<(np + 255) / 256, 256, 0, st>>>(dpairs, np, rep);
    }
    trace_mark(st, dir, "merge " + std::to_string(n_arcs) + " arcs, " + std::to_string(np) + " changed");
  }
  ::msc::count_launch();
  fill_i32_kernel<<<c.grid, 256, 0, st>>>(d.lab, N, -1);
  ::msc::count_launch();
  fill_i32_kernel<<<(n_ext + 256) / 256, 256, 0, st>>>(name, n_ext + 1, INT_MAX);
  LCUDA(cudaMemsetAsync(d.state, 0, (size_t)N, st), "memset");
  LCUDA(msc::launch_group_seeds(rep, d.seed, n_ext, name, d.lab, d.state, c.sms, st), "seeds");
  trace_mark(st, dir, "seeds");

  // certain terminal regions: a global frontier walk from the seeds to the fixpoint
  // (MSC_TERMINAL_TILES=1: tile passes instead)
  if (!terminal_tiles_on()) {
    int64_t* cur = c.list_a;
    int64_t* nxt = c.list_b;
    LCUDA(cudaMemcpyAsync(cur, d.seed, (size_t)n_ext * sizeof(int64_t), cudaMemcpyDeviceToDevice, st), "copy");
    int n = n_ext;
    std::memcpy(c.hpin, &n, sizeof(int));
    LCUDA(cudaMemcpyAsync(c.counters + 13, c.hpin, sizeof(int), cudaMemcpyHostToDevice, st), "write count");
    int* n_cur = c.counters + 13;
    int* n_nxt = c.counters + 14;
    int rounds = 0;
    while (n > 0) {
      if (rounds++ > N) return fail(MSC_ERR_ITER_LIMIT, "terminal regions did not converge");
      LCUDA(cudaMemsetAsync(n_nxt, 0, sizeof(int), st), "memset");
      LCUDA(msc::launch_terminal_walk(c.f, d.lab, V, dir, cur, n_cur, n, nxt, n_nxt, (int)N, c.counters + 4, c.sms, st),
            "regions");
      if (int rc = read_dev(c, n_nxt, 1, &n)) return rc;
      std::swap(cur, nxt);
      std::swap(n_cur, n_nxt);
    }
    trace_mark(st, dir, "terminal walk x" + std::to_string(rounds));
  } else {
  const uint8_t* din = nullptr;
  uint8_t* dout = c.tiles;
  for (int64_t passes = 0;; passes++) {
    LCUDA(cudaMemsetAsync(c.counters + 3, 0, sizeof(int), st), "memset");
    LCUDA(cudaMemsetAsync(dout, 0, (size_t)c.ntiles, st), "memset");
    LCUDA(msc::launch_terminal_pass(c.f, d.lab, V, dir, din, dout, c.counters + 3, c.counters + 4, c.sms, st),
          "regions");
    int changed = 0;
    if (int rc = read_dev(c, c.counters + 3, 1, &changed)) return rc;
    if (!changed) {
      trace_mark(st, dir, "terminal x" + std::to_string(passes + 1));
      break;
    }
    if (passes > c.ntiles + 2) return fail(MSC_ERR_ITER_LIMIT, "terminal regions did not converge");
    din = dout;
    dout = (dout == c.tiles) ? c.tiles + c.ntiles : c.tiles;
  }
  }
  if (stage_terminal) {
    ::msc::count_launch();
    snapshot_kernel<<<c.grid, 256, 0, st>>>(d.lab, stage_terminal, N);
  }
  ::msc::count_launch();
  terminal_state_kernel<<<c.grid, 256, 0, st>>>(d.lab, d.state, N);
  if (d.before_integration)
    if (int rc = d.before_integration()) return rc;
  return MSC_OK;
}

// Streamlines that orbit a sink of the interpolated gradient without reaching the
// stop threshold run to the iteration limit and end at their nearest vertex (on k^-3
// fields ~2% of the descending boundary re-decisions and 3/4 of their iterations).
// Outside the all-FP64 mode the integration kernels end such a streamline once it has
// stayed within 0.02 voxel for two windows of 64 iterations.  Where the orbit sits on a
// plane at which the nearest vertex changes, its final side is a coin flip of the
// chaotic orbit.  Against the all-FP64 labels (k^-3, asc / dsc): 3.6e-5 / 2.0e-4 of the
// vertices differ at 256^3, 3.8e-5 / 2.6e-4 at 192^3 (windows of 128: 3.4e-5 / 1.7e-4
// and 3.5e-5 / 2.1e-4, at 10% more time for the 512^3 labels).
msc::IntegParams integ_params(const msc_integ_params* p, int dir) {
  msc::IntegParams P{p->error_threshold, p->gradient_threshold, p->iteration_limit, (double)p->max_step, dir};
  if (p->precision != 1) {
    P.trap_window = 64;
    P.trap_radius = 0.02f;
  }
  return P;
}

// First integration pass of the vertices still unassigned (-1), after zeroing the
// gradient at this direction's seeds: the reference's spread order with one thread, run
// as batches (a group of levels, or part of one) of speculative streamlines whose
// resolution gives exactly the sequential outcome (integrate_kernels.cu).  A batch whose
// recorded sequences do not fit their pools is redone as two halves.
int first_pass(LabelCtx& c, DirLabels& d) {
  const int64_t N = c.N;
  cudaStream_t st = c.st;
  if (d.n_ext > 0 && !d.seeds_zeroed) {
    ::msc::count_launch();
    zero_seed_grad_kernel<<<(d.n_ext + 255) / 256, 256, 0, st>>>(d.seed, d.n_ext, c.g32, c.zeroed);
    d.seeds_zeroed = true;
  }
  const msc::IntegParams P = integ_params(c.p, d.dir);
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
  uint8_t* lvl;
  uint32_t* claim;
  int* counts;
  int32_t* vtx;
  uint32_t* ibits;
  unsigned long long* sc;  // [0] pool cursor [1] items [3] claimed items [4, 6) dirty-list lengths
                           // [6] holder-node cursor
  msc::SpecSet Q{};
  const int64_t max_items = std::min<int64_t>(N, S.offset[S.nlev]);
  const int64_t ibits_cap = max_items / 32 + 1;
  Q.pool_words = std::min<unsigned long long>(2ull * (unsigned long long)N + (1ull << 20), 0xFFFFFF00ull);
  Q.node_cap = std::min<unsigned long long>(3ull * (unsigned long long)N + (1ull << 20), 0x7FFFFF00ull);
  LCUDA(c.pool.get(&lvl, N), "alloc");
  LCUDA(c.pool.get(&claim, N), "alloc");
  LCUDA(c.pool.get(&counts, S.offset[S.nlev] / 1024 + 2), "alloc");
  LCUDA(c.pool.get(&vtx, max_items), "alloc");
  LCUDA(c.pool.get(&Q.e1, max_items), "alloc");
  LCUDA(c.pool.get(&Q.head, max_items), "alloc");
  LCUDA(c.pool.get(&Q.len, max_items), "alloc");
  LCUDA(c.pool.get(&Q.endlab, max_items), "alloc");
  LCUDA(c.pool.get(&Q.cut, max_items), "alloc");
  LCUDA(c.pool.get(&Q.ptr, max_items), "alloc");
  LCUDA(c.pool.get(&Q.alive, max_items), "alloc");
  LCUDA(c.pool.get(&Q.pool, Q.pool_words), "alloc");
  LCUDA(c.pool.get(&Q.hhead, N), "alloc");
  LCUDA(c.pool.get(&Q.hitem, Q.node_cap), "alloc");
  LCUDA(c.pool.get(&Q.hidx, Q.node_cap), "alloc");
  LCUDA(c.pool.get(&Q.hnext, Q.node_cap), "alloc");
  LCUDA(c.pool.get(&ibits, ibits_cap), "alloc");
  LCUDA(cudaMemsetAsync(ibits, 0, (size_t)ibits_cap * sizeof(uint32_t), st), "memset");  // (clear between rounds)
  LCUDA(c.pool.get(&sc, 8), "alloc");
  LCUDA(c.pool.get(&Q.overflow, 1), "alloc");
  msc::SpecDirty dirty[2];
  for (int q = 0; q < 2; q++) {
    dirty[q].words = N / 32 + 1;
    dirty[q].n = sc + 4 + q;
    LCUDA(c.pool.get(&dirty[q].bits, dirty[q].words), "alloc");
    LCUDA(cudaMemsetAsync(dirty[q].bits, 0, (size_t)dirty[q].words * sizeof(uint32_t), st), "memset");
    LCUDA(c.pool.get(&dirty[q].list, N), "alloc");
  }
  Q.vtx = vtx;
  Q.cursor = sc;
  Q.ncursor = sc + 6;
  // the vertices still unlabelled after a level (a byte scan): once there are none, the
  // remaining levels of the order hold no item (the last covers all N positions)
  unsigned long long* n_left;
  LCUDA(c.pool.get(&n_left, 1), "alloc");
  LCUDA(cudaMemsetAsync(claim, 0xFF, (size_t)N * sizeof(uint32_t), st), "memset");
  if (!d.trips_zeroed) {
    LCUDA(cudaMemsetAsync(c.work + 48, 0, 3 * sizeof(unsigned long long), st), "memset");
    d.trips_zeroed = true;
  }
  LCUDA(msc::launch_init_levels(d.lab, lvl, N, c.sms, st), "levels");
  trace_mark(st, d.dir, "pass1 start");
  // the levels up to N/512 visits together form the first batch; every later level is a
  // batch of its own
  const int64_t small = N / 512;
  int stamp = 0;
  int64_t rounds_total = 0, batches = 0;
  auto next_stamp = [&]() -> int {
    if (stamp >= 250) {  // stamps run out: every labelled vertex back to 0
      LCUDA(msc::launch_init_levels(d.lab, lvl, N, c.sms, st), "levels");
      stamp = 0;
    }
    ++stamp;
    return MSC_OK;
  };
  for (int L0 = 0; L0 < S.nlev;) {
    int L1 = L0 + 1;
    while (L1 < S.nlev && S.offset[L1 + 1] - S.offset[L0] <= small) L1++;
    const int64_t u0 = S.offset[L0], u1 = S.offset[L1];
    const int g0 = L0;
    L0 = L1;
    if (u1 <= u0) continue;
    if (int rc = next_stamp()) return rc;
    LCUDA(msc::launch_spread_compact(S, u0, u1, lvl, stamp, counts, vtx, sc + 1, st), "compact");
    unsigned long long n_items = 0;
    if (int rc = read_dev(c, sc + 1, 1, &n_items)) return rc;
    const int64_t n = (int64_t)n_items;
    for (int64_t k0 = 0; k0 < n;) {
      if (k0 > 0)
        if (int rc = next_stamp()) return rc;
      int64_t k1 = n;
      for (;;) {
        LCUDA(cudaMemsetAsync(sc, 0, sizeof(unsigned long long), st), "memset");
        LCUDA(cudaMemsetAsync(sc + 3, 0, sizeof(unsigned long long), st), "memset");
        LCUDA(cudaMemsetAsync(sc + 6, 0, sizeof(unsigned long long), st), "memset");
        LCUDA(cudaMemsetAsync(Q.hhead, 0xFF, (size_t)N * sizeof(int32_t), st), "memset");
        LCUDA(cudaMemsetAsync(Q.overflow, 0, sizeof(int), st), "memset");
        LCUDA(msc::launch_speculate(c.g32, c.V, P, Q, k0, k1, d.lab, lvl, stamp, claim, sc + 3, c.work + 48, c.sms,
                                    st),
              "speculate");
        int ovf = 0;
        if (int rc = read_dev(c, Q.overflow, 1, &ovf)) return rc;
        if (!ovf) break;
        LCUDA(msc::launch_spec_unclaim_all(lvl, stamp, claim, N, c.sms, st), "unclaim");
        if (k1 - k0 <= 1) return fail(MSC_ERR_OOM, "first pass: one streamline's record exceeds its pool");
        k1 = k0 + (k1 - k0) / 2;
      }
      trace_mark(st, d.dir, "  speculated " + std::to_string(k1 - k0));
      // resolution rounds: the first looks at every item, a later one at the items that
      // hold a vertex whose claim may have changed; they end when a round changes no
      // claim.  After the first two, rounds go in groups of four between counter reads
      // (a round after the last one finds nothing to do).
      for (int64_t r = 0;;) {
        if (r > k1 - k0 + 8) return fail(MSC_ERR_ITER_LIMIT, "first-pass resolution did not converge");
        const int group = r < 2 ? 1 : 4;
        for (int q = 0; q < group; q++, r++)
          LCUDA(msc::launch_spec_round(Q, k0, k1, claim, r == 0 ? nullptr : &dirty[r & 1], dirty[(r + 1) & 1], ibits,
                                       (k1 - k0) / 32 + 1, c.sms, st),
                "resolve");
        unsigned long long nd = 0;
        if (int rc = read_dev(c, dirty[r & 1].n, 1, &nd)) return rc;
        rounds_total += group;
        if (r == 1) trace_mark(st, d.dir, "  round 1: " + std::to_string(nd) + " dirty");
        if (nd == 0) break;
      }
      trace_mark(st, d.dir, "  resolved");
      LCUDA(msc::launch_spec_ptr(Q, k0, k1, claim, c.sms, st), "label");
      LCUDA(cudaMemsetAsync(Q.overflow, 0, sizeof(int), st), "memset");
      LCUDA(msc::launch_spec_write(Q, k0, k1, lvl, stamp, claim, d.lab, Q.overflow, c.sms, st), "label");
      int long_chain = 0;
      if (int rc = read_dev(c, Q.overflow, 1, &long_chain)) return rc;
      if (long_chain) {  // a few long chains of cut items: jump, then write again
        LCUDA(msc::launch_spec_jumps(Q, k0, k1, c.sms, st), "label");
        LCUDA(msc::launch_spec_write(Q, k0, k1, lvl, stamp, claim, d.lab, Q.overflow, c.sms, st), "label");
      }
      batches++;
      trace_mark(st, d.dir, "batch " + std::to_string(g0) + "-" + std::to_string(L1 - 1) + " items " +
                                std::to_string(k1 - k0) + " rounds " + std::to_string(rounds_total));
      k0 = k1;
    }
    LCUDA(msc::launch_count_unlabelled(lvl, N, n_left, c.sms, st), "count");
    unsigned long long left = 0;
    if (int rc = read_dev(c, n_left, 1, &left)) return rc;
    if (left == 0) break;  // every vertex labelled
  }
  trace_mark(st, d.dir, "pass1 (" + std::to_string(batches) + " batches, " + std::to_string(rounds_total) + " rounds)");
  return MSC_OK;
}

// Boundary fix-up of the vertices still marked unassigned in d.state, then the
// cleaner; `out` receives the final labels.
struct EarlyEnds {
  bool on = false;
  int32_t* endv = nullptr;
  int64_t* list = nullptr;
};

int finish_direction(LabelCtx& c, DirLabels& d, int32_t* out, int32_t* stage_integrated, int64_t stats[2],
                     const EarlyEnds* early = nullptr) {
  const int64_t N = c.N;
  const msc::VolDims& V = c.V;
  cudaStream_t st = c.st;
  const msc_integ_params* p = c.p;
  const int sms = c.sms;
  const msc::IntegParams P = integ_params(p, d.dir);

  // fix-up waves until no decision reopens a neighbour (:316-415).  Each wave first
  // integrates its members that have no streamline end yet -- in FP32, and the ones whose
  // FP32 ending is ambiguous again in FP64 (or all in FP64: precision 1) -- then decides
  // the wave in the reference's one-thread order (integrate_kernels.cu, wave kernels).
  // An end does not depend on labels, so a vertex decided in several waves integrates
  // once.
  int32_t *endv, *inw, *rptr, *rval, *rfin;
  LCUDA(c.pool.get(&rfin, N), "alloc");
  LCUDA(c.pool.get(&inw, N), "alloc");
  LCUDA(c.pool.get(&rptr, N), "alloc");
  LCUDA(c.pool.get(&rval, N), "alloc");
  int64_t early_n = 0, early_amb = 0;
  if (early) {
    // the ends computed beside the first pass (FP32, and FP64 where the FP32 ending was
    // ambiguous)
    endv = early->endv;
    LCUDA(cudaStreamWaitEvent(st, c.ends_done, 0), "cudaStreamWaitEvent");
    int h[2] = {0, 0};
    if (int rc = read_dev(c, c.counters + 7, 1, &h[0])) return rc;
    if (int rc = read_dev(c, c.counters + 12, 1, &h[1])) return rc;
    trace_mark(st, d.dir, "ends of " + std::to_string(h[1]) + " (FP64 " + std::to_string(h[0]) + ")");
    early_amb = h[0];
    early_n = h[1];
  } else {
    LCUDA(c.pool.get(&endv, N), "alloc");
    LCUDA(cudaMemsetAsync(endv, 0xFF, N * sizeof(int32_t), st), "memset");
  }
  LCUDA(cudaMemsetAsync(inw, 0xFF, N * sizeof(int32_t), st), "memset");
  LCUDA(cudaMemsetAsync(c.queued, 0, (N / 32 + 1) * sizeof(uint32_t), st), "memset");
  LCUDA(cudaMemsetAsync(c.counters + 5, 0, 3 * sizeof(int), st), "memset");
  LCUDA(msc::launch_boundary_set(d.lab, d.state, V, c.list_a, c.counters + 5, c.queued, sms, st), "boundary set");
  int n_list = 0;
  if (int rc = read_dev(c, c.counters + 5, 1, &n_list)) return rc;
  trace_mark(st, d.dir, "boundary " + std::to_string(n_list));
  if (p->precision == 3) n_list = 0;  // first pass only
  int64_t* cur = c.list_a;
  int64_t* nxt = c.list_b;
  int64_t* todo = c.list_c;
  stats[0] = early_n;
  stats[1] = early_amb;
  for (int w = 0; n_list > 0; w++) {
    if (w > 2 * N + 2) return fail(MSC_ERR_ITER_LIMIT, "fix-up did not converge");
    // counters: [5] todo, [6] next wave, [7] ambiguous
    LCUDA(cudaMemsetAsync(c.counters + 5, 0, 3 * sizeof(int), st), "memset");
    LCUDA(msc::launch_wave_mark(cur, n_list, w, inw, c.queued, endv, todo, c.counters + 5, sms, st), "wave");
    int n_todo = 0;
    if (int rc = read_dev(c, c.counters + 5, 1, &n_todo)) return rc;
    int n_amb = 0;
    if (p->precision == 1) {
      n_amb = n_todo;
      LCUDA(msc::launch_fixup_end64(c.f, c.zeroed, V, P, d.state, todo, n_todo, endv, c.work, c.work + 50, sms, st),
            "fix-up");
    } else if (n_todo > 0) {
      LCUDA(msc::launch_fixup_end32(c.g32, V, P, d.lab, d.state, todo, n_todo, endv, c.amb, c.counters + 7,
                                    p->precision == 2 ? 2 : 0, c.work, c.work + 49, sms, st),
            "fix-up");
      if (int rc = read_dev(c, c.counters + 7, 1, &n_amb)) return rc;
      trace_mark(st, d.dir, "  fp32 ends");
      LCUDA(msc::launch_fixup_end64(c.f, c.zeroed, V, P, d.state, c.amb, n_amb, endv, c.work + 56, c.work + 50, sms,
                                    st),
            "fix-up FP64");
      trace_mark(st, d.dir, "  fp64 ends");
    }
    stats[0] += n_todo;
    stats[1] += n_amb;
    int long_chain = 0;
    LCUDA(msc::launch_wave_resolve(cur, n_list, w, endv, inw, d.lab, d.state, rptr, rval, rfin, c.counters + 10, false,
                                   sms, st),
          "wave decide");
    if (int rc = read_dev(c, c.counters + 10, 1, &long_chain)) return rc;
    if (long_chain)
      LCUDA(msc::launch_wave_resolve(cur, n_list, w, endv, inw, d.lab, d.state, rptr, rval, rfin, c.counters + 10,
                                     true, sms, st),
            "wave decide");
    LCUDA(msc::launch_wave_finish(cur, n_list, w, V, rfin, inw, d.lab, d.state, c.queued, nxt, c.counters + 6, sms, st),
          "wave decide");
    if (int rc = read_dev(c, c.counters + 6, 1, &n_list)) return rc;
    std::swap(cur, nxt);
    trace_mark(st, d.dir, "wave " + std::to_string(w) + " integrated " + std::to_string(n_todo) + " (FP64 " +
                              std::to_string(n_amb) + ") next " + std::to_string(n_list));
  }
  {
    unsigned long long h[3];
    if (int rc = read_dev(c, c.work + 48, 3, h)) return rc;
    for (int k = 0; k < 3; k++) d.trips[k] = (int64_t)h[k];
  }
  if (stage_integrated) {
    ::msc::count_launch();
    snapshot_kernel<<<c.grid, 256, 0, st>>>(d.lab, stage_integrated, N);
  }
  if (!out) return MSC_OK;

  // isolated-region cleaner
  int32_t *parent, *first, *md, *roots;  // (fewer than 2^31 vertices: setup_ctx)
  LCUDA(c.pool.get(&parent, N), "alloc");
  LCUDA(c.pool.get(&first, N), "alloc");
  LCUDA(c.pool.get(&md, N), "alloc");
  LCUDA(c.pool.get(&roots, N), "alloc");
  int sweeps = 0;
  LCUDA(msc::launch_clean(d.lab, c.f, V, d.dir, parent, first, md, roots, c.counters + 8,
                          reinterpret_cast<int*>(c.hpin), out, sms, st, &sweeps),
        "clean");
  trace_mark(st, d.dir, "clean (" + std::to_string(sweeps) + " sweeps)");
  return MSC_OK;
}

// Every fix-up streamline ends where it reaches a certain terminal region (or stops),
// whatever the labels, and the certain terminals are known before the first pass.  So
// the ends of all the vertices a wave can hold -- those that are not certain terminals
// -- are computed in one launch on a stream of their own while the first pass runs:
// the waves then only decide.  A wave that integrated its own members would end with
// the slowest of its streamlines, ten waves and more per direction; one launch over
// all of them keeps only the one longest streamline in the tail, and the launch fills
// the gaps the first pass leaves (its resolution rounds are small launches between
// host reads).  The extra ends (vertices no wave takes) cost about a fifth more
// integration.  MSC_EARLY_ENDS=0 integrates per wave instead.
bool early_ends_on() {
  static const bool on = [] {
    const char* e = std::getenv("MSC_EARLY_ENDS");
    return !(e && std::atoi(e) == 0);
  }();
  return on;
}

int start_early_ends(LabelCtx& c, DirLabels& d, EarlyEnds& e) {
  const int64_t N = c.N;
  cudaStream_t st = c.st;
  LCUDA(c.pool.get(&e.endv, N), "alloc");
  LCUDA(c.pool.get(&e.list, N), "alloc");
  LCUDA(cudaMemsetAsync(e.endv, 0xFF, N * sizeof(int32_t), st), "memset");
  LCUDA(cudaMemsetAsync(c.counters + 12, 0, sizeof(int), st), "memset");
  LCUDA(cudaMemsetAsync(c.counters + 7, 0, sizeof(int), st), "memset");
  // the iteration counters before the ends launch adds to them (the first pass leaves
  // them alone then)
  LCUDA(cudaMemsetAsync(c.work + 48, 0, 3 * sizeof(unsigned long long), st), "memset");
  d.trips_zeroed = true;
  // the streamlines see the gradient the first pass sees: zero at this direction's seeds
  if (d.n_ext > 0 && !d.seeds_zeroed) {
    ::msc::count_launch();
    zero_seed_grad_kernel<<<(d.n_ext + 255) / 256, 256, 0, st>>>(d.seed, d.n_ext, c.g32, c.zeroed);
    d.seeds_zeroed = true;
  }
  if (!c.ends_st) {
    LCUDA(cudaStreamCreateWithFlags(&c.ends_st, cudaStreamNonBlocking), "cudaStreamCreate");
    LCUDA(cudaEventCreateWithFlags(&c.ends_go, cudaEventDisableTiming), "cudaEventCreate");
    LCUDA(cudaEventCreateWithFlags(&c.ends_done, cudaEventDisableTiming), "cudaEventCreate");
  }
  LCUDA(cudaEventRecord(c.ends_go, st), "cudaEventRecord");
  LCUDA(cudaStreamWaitEvent(c.ends_st, c.ends_go, 0), "cudaStreamWaitEvent");
  const msc::IntegParams P = integ_params(c.p, d.dir);
  LCUDA(msc::launch_uncertain_list(d.state, N, e.list, c.counters + 12, c.sms, c.ends_st), "fix-up candidates");
  LCUDA(msc::launch_fixup_end32(c.g32, c.V, P, d.lab, d.state, e.list, (int)N, e.endv, c.amb, c.counters + 7,
                                c.p->precision == 2 ? 2 : 0, c.work, c.work + 49, c.sms, c.ends_st, c.counters + 12),
        "fix-up ends");
  // and in FP64 the ones whose FP32 ending was ambiguous (their count stays on the device)
  LCUDA(msc::launch_fixup_end64(c.f, c.zeroed, c.V, P, d.state, c.amb, 1, e.endv, c.work + 56, c.work + 50, c.sms,
                                c.ends_st, c.counters + 7),
        "fix-up FP64 ends");
  LCUDA(cudaEventRecord(c.ends_done, c.ends_st), "cudaEventRecord");
  e.on = true;
  return MSC_OK;
}

int integrate_direction(LabelCtx& c, DirLabels& d, int32_t* out, int32_t* stage_integrated, int64_t stats[2]) {
  EarlyEnds e;
  if (early_ends_on() && (c.p->precision == 0 || c.p->precision == 2))
    if (int rc = start_early_ends(c, d, e)) return rc;
  if (int rc = first_pass(c, d)) return rc;
  return finish_direction(c, d, out, stage_integrated, stats, e.on ? &e : nullptr);
}

int finish_errors(LabelCtx& c) {
  int err = 0;
  if (int rc = read_dev(c, c.counters + 4, 1, &err)) return rc;
  if (err & msc::kErrLocalQueue) return fail(MSC_ERR_QUEUE_OVERFLOW, "tile queue overflow");
  if (err & msc::kErrIterLimit) return fail(MSC_ERR_ITER_LIMIT, "V-path walk exceeded its bound (invalid gradient?)");
  return MSC_OK;
}

int labels_concurrent(const float* f, const uint8_t* grad, const int64_t* dims, const msc_integ_params* p,
                      const msc_triage_params* tp, int32_t* out_asc, int32_t* out_dsc, int32_t* stages,
                      int64_t* tstats, cudaStream_t st);
int direction_rest(LabelCtx& c, DirLabels& d, int k, const msc_triage_params* tp, int32_t* out,
                   int32_t* stage_integrated, int64_t fix[2], int64_t counts_out[3]);

// The descending direction of a two-direction call on its own stream and host thread,
// concurrently with the ascending one: the two share nothing but the inputs, so their
// kernels fill each other's idle time (launch tails, host synchronisation, the FP64
// re-decisions).  The reference integrates the descending labels on the gradient the
// ascending pass zeroed at the minima' seeds; this job has its own gradient copy and
// zeroes those seeds too once the ascending job has found them (`asc_seeds`).
struct SeedHandoff {
  std::mutex mu;
  std::condition_variable cv;
  bool ready = false;
  const int64_t* seed = nullptr;  // device, on the ascending job's stream
  int n = -1;                     // -1: the ascending job failed before its seeds
  cudaEvent_t done = nullptr;     // recorded on the ascending stream after the seeds
  void publish(const int64_t* s, int k, cudaEvent_t e) {
    std::lock_guard<std::mutex> lk(mu);
    seed = s;
    n = k;
    done = e;
    ready = true;
    cv.notify_all();
  }
};

struct DscJob {
  int rc = MSC_OK;
  std::string err;
  int64_t stats[2] = {0, 0};
  int64_t trips[3] = {0, 0, 0};
  int64_t counts[3] = {0, 0, 0};  // triage: flagged, audited, audited the fix-up changed
};

void run_dsc_job(int dev, cudaEvent_t inputs_ready, const float* f, const uint8_t* grad, const int64_t* dims,
                 const msc_integ_params* p, const msc_triage_params* tp, int32_t* out, int32_t* stages,
                 SeedHandoff* asc, DscJob* job) {
  auto body = [&]() -> int {
    LCUDA(cudaSetDevice(dev), "cudaSetDevice");
    cudaStream_t sb = nullptr;
    // the descending labels take about twice the ascending ones' work (their streamlines
    // are longer), so their stream goes first where both have blocks waiting
    // (MSC_DSC_PRIORITY=0: the default priority)
    int lo = 0, hi = 0;
    LCUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi), "cudaDeviceGetStreamPriorityRange");
    static const bool prio = [] {
      const char* e = std::getenv("MSC_DSC_PRIORITY");
      return !(e && std::atoi(e) == 0);
    }();
    LCUDA(cudaStreamCreateWithPriority(&sb, cudaStreamNonBlocking, prio ? hi : lo), "cudaStreamCreate");
    struct Destroy {
      cudaStream_t s;
      ~Destroy() {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
      }
    } ds{sb};
    LCUDA(cudaStreamWaitEvent(sb, inputs_ready, 0), "cudaStreamWaitEvent");
    int rc = MSC_OK;
    {
      trace_mark(sb, 1, "start");
      LabelCtx c(sb);
      if ((rc = setup_ctx(c, f, grad, dims, p))) return rc;
      trace_mark(sb, 1, "setup");
      DirLabels d;
      d.dir = 1;
      // the ascending job's seeds, zeroed in this direction's gradient before its
      // streamlines start (the terminal regions before them do not read the gradient, and
      // grow while the ascending job merges its extrema)
      d.before_integration = [&]() -> int {
        {
          std::unique_lock<std::mutex> lk(asc->mu);
          asc->cv.wait(lk, [&] { return asc->ready; });
        }
        if (asc->n < 0) return fail(MSC_ERR_CUDA, "ascending labels failed");
        if (asc->n > 0) {
          LCUDA(cudaStreamWaitEvent(sb, asc->done, 0), "cudaStreamWaitEvent");
          ::msc::count_launch();
          zero_seed_grad_kernel<<<(asc->n + 255) / 256, 256, 0, sb>>>(asc->seed, asc->n, c.g32, c.zeroed);
        }
        trace_mark(sb, 1, "asc seeds zeroed");
        return MSC_OK;
      };
      if ((rc = prepare_direction(c, d, stages ? stages + 2 * c.N : nullptr))) return rc;
      if ((rc = direction_rest(c, d, 1, tp, out, stages ? stages + 3 * c.N : nullptr, job->stats, job->counts)))
        return rc;
      for (int k = 0; k < 3; k++) job->trips[k] = d.trips[k];
      rc = finish_errors(c);
    }
    return rc;
  };
  job->rc = body();
  if (job->rc != MSC_OK) job->err = t_err;
}

int labels_impl(const float* f, const uint8_t* grad, const int64_t* dims, const msc_integ_params* p, int32_t* out_asc,
                int32_t* out_dsc, int32_t* stages, cudaStream_t st) {
  if (!out_asc && !out_dsc) return fail(MSC_ERR_NULL_POINTER, "null argument");
  if (out_asc && out_dsc) return labels_concurrent(f, grad, dims, p, nullptr, out_asc, out_dsc, stages, nullptr, st);
  LabelCtx c(st);
  if (int rc = setup_ctx(c, f, grad, dims, p)) return rc;
  for (int k = 0; k < 4; k++) t_stats[k] = 0;
  for (int k = 0; k < 6; k++) t_trips[k] = 0;
  for (int pass = 0; pass < 2; pass++) {
    int32_t* out = pass == 0 ? out_asc : out_dsc;
    if (!out) continue;
    DirLabels d;
    d.dir = pass == 0 ? -1 : 1;
    if (int rc = prepare_direction(c, d, stages ? stages + (2 * pass) * c.N : nullptr)) return rc;
    if (int rc = integrate_direction(c, d, out, stages ? stages + (2 * pass + 1) * c.N : nullptr, t_stats + 2 * pass))
      return rc;
    for (int k = 0; k < 3; k++) t_trips[3 * pass + k] = d.trips[k];
  }
  const int rc = finish_errors(c);
  trace_dump();
  return rc;
}

// Both directions: the ascending one on the caller's stream and thread, the
// descending one concurrently (run_dsc_job).
int labels_concurrent(const float* f, const uint8_t* grad, const int64_t* dims, const msc_integ_params* p,
                      const msc_triage_params* tp, int32_t* out_asc, int32_t* out_dsc, int32_t* stages,
                      int64_t* tstats, cudaStream_t st) {
  for (int k = 0; k < 4; k++) t_stats[k] = 0;
  for (int k = 0; k < 6; k++) t_trips[k] = 0;
  int dev = 0;
  LCUDA(cudaGetDevice(&dev), "cudaGetDevice");
  cudaEvent_t inputs_ready = nullptr, seeds_done = nullptr;
  LCUDA(cudaEventCreateWithFlags(&inputs_ready, cudaEventDisableTiming), "cudaEventCreate");
  LCUDA(cudaEventCreateWithFlags(&seeds_done, cudaEventDisableTiming), "cudaEventCreate");
  struct Events {
    cudaEvent_t a, b;
    ~Events() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } evs{inputs_ready, seeds_done};
  LCUDA(cudaEventRecord(inputs_ready, st), "cudaEventRecord");
  SeedHandoff handoff;
  DscJob job;
  std::thread worker;
  try {
    worker = std::thread(run_dsc_job, dev, inputs_ready, f, grad, dims, p, tp, out_dsc, stages, &handoff, &job);
  } catch (...) {
    return fail(MSC_ERR_CUDA, "could not start the descending labels' host thread");
  }
  int rc = MSC_OK;
  int64_t counts[3] = {0, 0, 0};
  {
    trace_mark(st, -1, "start");
    LabelCtx c(st);
    DirLabels d;
    d.dir = -1;
    // the minima' seeds go to run_dsc_job (which zeroes them in its gradient copy) as
    // soon as they exist, before this direction's extremum merge and terminal regions
    bool published = false;
    d.on_seeds = [&]() -> int {
      LCUDA(cudaEventRecord(seeds_done, st), "cudaEventRecord");
      handoff.publish(d.seed, d.n_ext, seeds_done);
      published = true;
      return MSC_OK;
    };
    rc = setup_ctx(c, f, grad, dims, p);
    trace_mark(st, -1, "setup");
    if (rc == MSC_OK) rc = prepare_direction(c, d, stages);
    if (!published) handoff.publish(nullptr, -1, nullptr);
    if (rc == MSC_OK) rc = direction_rest(c, d, 0, tp, out_asc, stages ? stages + c.N : nullptr, t_stats, counts);
    for (int k = 0; k < 3; k++) t_trips[k] = d.trips[k];
    if (rc == MSC_OK) rc = finish_errors(c);
    // the descending job reads d.seed from this context's pool: wait for it first
    worker.join();
  }
  trace_dump();
  if (rc != MSC_OK) return rc;
  if (job.rc != MSC_OK) return fail(job.rc, job.err);
  t_stats[2] = job.stats[0];
  t_stats[3] = job.stats[1];
  for (int k = 0; k < 3; k++) t_trips[3 + k] = job.trips[k];
  if (tstats) {
    for (int k = 0; k < 3; k++) {
      tstats[k] = counts[k];
      tstats[4 + k] = job.counts[k];
    }
    tstats[3] = t_stats[0];
    tstats[7] = t_stats[2];
  }
  return MSC_OK;
}

// Network features of one direction from its first-pass labels (triage_prep.cu).
int direction_features(LabelCtx& c, DirLabels& d, __nv_bfloat16* feat) {
  double* sums;
  LCUDA(c.pool.get(&sums, 3), "alloc");
  LCUDA(msc::launch_features(c.f, c.g32, d.lab, d.state, c.V, d.dir, sums, feat, c.sms, c.st), "features");
  return MSC_OK;
}

// Training data: per direction, the features after the first pass and the targets
// (1 where the full boundary fix-up changes the first-pass label).  The directions
// run one after the other, as the plain labeling does.
int triage_features_impl(const float* f, const uint8_t* grad, const int64_t* dims, const msc_integ_params* p,
                         uint16_t* features, uint8_t* targets, cudaStream_t st) {
  if (!features) return fail(MSC_ERR_NULL_POINTER, "null argument");
  LabelCtx c(st);
  if (int rc = setup_ctx(c, f, grad, dims, p)) return rc;
  const int64_t N = c.N;
  int32_t* first;
  LCUDA(c.pool.get(&first, N), "alloc");
  for (int k = 0; k < 2; k++) {
    DirLabels d;
    d.dir = k == 0 ? -1 : 1;
    if (int rc = prepare_direction(c, d, nullptr)) return rc;
    if (int rc = first_pass(c, d)) return rc;
    if (int rc = direction_features(c, d, reinterpret_cast<__nv_bfloat16*>(features) + (size_t)k * 16 * N)) return rc;
    if (targets) {
      LCUDA(cudaMemcpyAsync(first, d.lab, N * sizeof(int32_t), cudaMemcpyDeviceToDevice, st), "copy");
      int64_t fx[2];
      if (int rc = finish_direction(c, d, nullptr, nullptr, fx)) return rc;
      LCUDA(msc::launch_change_targets(d.lab, first, N, targets + (size_t)k * 2 * N, c.sms, st), "targets");
    }
  }
  return finish_errors(c);
}

// After prepare_direction: the plain rest of one direction (first pass, fix-up,
// cleaner) or, with `tp`, the triaged one -- first pass, network features and
// inference, the flagged vertices plus the audit into the fix-up, the audit count.
// k: 0 ascending, 1 descending; counts_out (triage): flagged, audited, audited the
// fix-up changed.
int direction_rest(LabelCtx& c, DirLabels& d, int k, const msc_triage_params* tp, int32_t* out,
                   int32_t* stage_integrated, int64_t fix[2], int64_t counts_out[3]) {
  if (!tp) return integrate_direction(c, d, out, stage_integrated, fix);
  cudaStream_t st = c.st;
  const int64_t N = c.N;
  uint8_t *blobs, *flags;
  __nv_bfloat16 *feat, *act1, *act2;
  float* logits;
  int32_t* first;
  unsigned long long* counts;
  LCUDA(c.pool.get(&blobs, msc::kTriageBlobBytes), "alloc");
  LCUDA(c.pool.get(&feat, 16 * N), "alloc");
  LCUDA(c.pool.get(&act1, 16 * N), "alloc");
  LCUDA(c.pool.get(&act2, 16 * N), "alloc");
  LCUDA(c.pool.get(&logits, 2 * N), "alloc");
  LCUDA(c.pool.get(&flags, N), "alloc");
  LCUDA(c.pool.get(&first, N), "alloc");
  LCUDA(c.pool.get(&counts, 3), "alloc");
  LCUDA(cudaMemsetAsync(counts, 0, 3 * sizeof(unsigned long long), st), "memset");
  const msc::ConvDims D{c.V.X, c.V.Y, c.V.Z, N};
  const float thr = k == 0 ? tp->logit_threshold_asc : tp->logit_threshold_dsc;
  if (int rc = first_pass(c, d)) return rc;
  if (int rc = direction_features(c, d, feat)) return rc;
  LCUDA(msc::triage_forward(feat, D, tp->weights, blobs, act1, act2, logits, c.counters + 4, st), "triage forward");
  LCUDA(cudaMemcpyAsync(first, d.lab, N * sizeof(int32_t), cudaMemcpyDeviceToDevice, st), "copy");
  LCUDA(msc::launch_triage_apply(logits, thr, d.state, flags, N, tp->audit_fraction, tp->audit_seed + (uint64_t)k,
                                 counts, c.sms, st),
        "triage apply");
  if (int rc = finish_direction(c, d, out, nullptr, fix)) return rc;
  LCUDA(msc::launch_audit_count(d.lab, first, flags, N, counts + 2, c.sms, st), "audit");
  unsigned long long h[3];
  if (int rc = read_dev(c, counts, 3, h)) return rc;
  for (int q = 0; q < 3; q++) counts_out[q] = (int64_t)h[q];
  return MSC_OK;
}

// Both directions with triage, concurrently (labels_concurrent).
int triage_labels_impl(const float* f, const uint8_t* grad, const int64_t* dims, const msc_integ_params* p,
                       const msc_triage_params* tp, int32_t* out_asc, int32_t* out_dsc, int64_t* stats,
                       cudaStream_t st) {
  if (!out_asc || !out_dsc || !tp || !tp->weights) return fail(MSC_ERR_NULL_POINTER, "null argument");
  int64_t tstats[8];
  if (int rc = labels_concurrent(f, grad, dims, p, tp, out_asc, out_dsc, nullptr, tstats, st)) return rc;
  if (stats)
    for (int k = 0; k < 8; k++) stats[k] = tstats[k];
  return MSC_OK;
}

// Per-thread device staging of the host-buffer entry, kept between calls.
struct LabelStaging {
  int dev = -1;
  cudaStream_t st = nullptr;
  size_t nv = 0, nc = 0;
  float* f = nullptr;
  uint8_t* g = nullptr;
  int32_t* lab = nullptr;  // [2][N]
};
thread_local LabelStaging t_lstage;

int labels_host_impl(const float* fh, const int64_t* dims, const msc_integ_params* p, const msc_triage_params* tp,
                     int32_t* asc_h, int32_t* dsc_h) {
  if (!fh || !dims || !p || !asc_h || !dsc_h) return fail(MSC_ERR_NULL_POINTER, "null argument");
  if (dims[0] < 2 || dims[1] < 2 || dims[2] < 2) return fail(MSC_ERR_BAD_DIMS, "labeling needs 2 <= X, Y, Z");
  const size_t nv = (size_t)(dims[0] * dims[1] * dims[2]);
  const int64_t nc64 = msc_num_cells_3d(dims);
  if (nc64 < 0) return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  const size_t nc = (size_t)nc64;
  int dev = 0;
  LCUDA(cudaGetDevice(&dev), "cudaGetDevice");
  LabelStaging& h = t_lstage;
  if (h.dev != dev) {
    h = LabelStaging{};
    h.dev = dev;
  }
  if (!h.st) LCUDA(cudaStreamCreateWithFlags(&h.st, cudaStreamNonBlocking), "cudaStreamCreate");
  if (h.nv < nv) {
    if (h.f) cudaFree(h.f);
    if (h.lab) cudaFree(h.lab);
    h.f = nullptr;
    h.lab = nullptr;
    h.nv = 0;
    LCUDA(cudaMalloc((void**)&h.f, nv * sizeof(float)), "cudaMalloc(f staging)");
    LCUDA(cudaMalloc((void**)&h.lab, 2 * nv * sizeof(int32_t)), "cudaMalloc(label staging)");
    h.nv = nv;
  }
  if (h.nc < nc) {
    if (h.g) cudaFree(h.g);
    h.g = nullptr;
    h.nc = 0;
    LCUDA(cudaMalloc((void**)&h.g, nc), "cudaMalloc(grad staging)");
    h.nc = nc;
  }
  LCUDA(cudaMemcpyAsync(h.f, fh, nv * sizeof(float), cudaMemcpyHostToDevice, h.st), "copy f to device");
  if (int rc = msc_lower_star_grad_3d(h.f, dims, h.g, h.st)) return fail(rc, msc_last_error_string());
  int rc = tp ? triage_labels_impl(h.f, h.g, dims, p, tp, h.lab, h.lab + nv, nullptr, h.st)
              : labels_impl(h.f, h.g, dims, p, h.lab, h.lab + nv, nullptr, h.st);
  if (rc) return rc;
  LCUDA(cudaMemcpyAsync(asc_h, h.lab, nv * sizeof(int32_t), cudaMemcpyDeviceToHost, h.st), "copy labels to host");
  LCUDA(cudaMemcpyAsync(dsc_h, h.lab + nv, nv * sizeof(int32_t), cudaMemcpyDeviceToHost, h.st), "copy labels to host");
  LCUDA(cudaStreamSynchronize(h.st), "cudaStreamSynchronize");
  return MSC_OK;
}

// The cleaner alone on caller labels (msc_clean_regions_3d).
int clean_impl(const float* f, const int32_t* labels_in, const int64_t* dims, int direction, int32_t* labels_out,
               cudaStream_t st) {
  if (!f || !labels_in || !labels_out || !dims) return fail(MSC_ERR_NULL_POINTER, "null argument");
  if (direction != -1 && direction != 1) return fail(MSC_ERR_BAD_DIMS, "direction must be -1 or +1");
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1 || dims[0] > (1 << 30) || dims[1] > (1 << 30) || dims[2] > (1 << 30))
    return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  const int64_t N = dims[0] * dims[1] * dims[2];
  if (N / dims[2] != dims[0] * dims[1] || N >= ((int64_t)1 << 31)) return fail(MSC_ERR_BAD_DIMS, "fewer than 2^31 vertices");
  LabelCtx c(st);
  if (!(c.hpin = pinned_get())) return fail(MSC_ERR_OOM, "pinned host words");
  const msc::VolDims V{dims[0], dims[1], dims[2], 2 * dims[0] - 1, 2 * dims[1] - 1, 2 * dims[2] - 1,
                       2 * dims[0] - 1, (2 * dims[0] - 1) * (2 * dims[1] - 1)};
  const int sms = sm_count();
  int32_t *lab, *parent, *first, *md, *roots;
  int* counters;
  LCUDA(c.pool.get(&lab, N), "alloc");
  LCUDA(c.pool.get(&parent, N), "alloc");
  LCUDA(c.pool.get(&first, N), "alloc");
  LCUDA(c.pool.get(&md, N), "alloc");
  LCUDA(c.pool.get(&roots, N), "alloc");
  LCUDA(c.pool.get(&counters, 2), "alloc");
  ::msc::count_launch();
  none_in_kernel<<<sms * 8, 256, 0, st>>>(labels_in, lab, N);
  LCUDA(msc::launch_clean(lab, f, V, direction, parent, first, md, roots, counters, reinterpret_cast<int*>(c.hpin),
                          labels_out, sms, st, nullptr),
        "clean");
  LCUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  return MSC_OK;
}

}  // namespace

extern "C" {

int msc_clean_regions_3d(const float* f, const int32_t* labels_in, const int64_t dims[3], int direction,
                         int32_t* labels_out, msc_stream_t stream) {
  return clean_impl(f, labels_in, dims, direction, labels_out, (cudaStream_t)stream);
}


const char* msc_labels_last_error_string(void) { return t_err.c_str(); }

void msc_labels_last_stats(int64_t out[4]) {
  if (out)
    for (int k = 0; k < 4; k++) out[k] = t_stats[k];
}

void msc_labels_last_iterations(int64_t out[6]) {
  if (out)
    for (int k = 0; k < 6; k++) out[k] = t_trips[k];
}

int msc_integrated_labels_3d(const float* f, const uint8_t* grad, const int64_t dims[3], const msc_integ_params* params,
                             int32_t* labels_asc, int32_t* labels_dsc, msc_stream_t stream) {
  return labels_impl(f, grad, dims, params, labels_asc, labels_dsc, nullptr, (cudaStream_t)stream);
}

int msc_integrated_labels_3d_stages(const float* f, const uint8_t* grad, const int64_t dims[3],
                                    const msc_integ_params* params, int32_t* labels_asc, int32_t* labels_dsc,
                                    int32_t* stages, msc_stream_t stream) {
  return labels_impl(f, grad, dims, params, labels_asc, labels_dsc, stages, (cudaStream_t)stream);
}

int msc_triage_features_3d(const float* f, const uint8_t* grad, const int64_t dims[3], const msc_integ_params* params,
                           uint16_t* features, uint8_t* targets, msc_stream_t stream) {
  return triage_features_impl(f, grad, dims, params, features, targets, (cudaStream_t)stream);
}

int msc_triage_labels_3d(const float* f, const uint8_t* grad, const int64_t dims[3], const msc_integ_params* params,
                         const msc_triage_params* triage, int32_t* labels_asc, int32_t* labels_dsc, int64_t stats[8],
                         msc_stream_t stream) {
  return triage_labels_impl(f, grad, dims, params, triage, labels_asc, labels_dsc, stats, (cudaStream_t)stream);
}

int msc_ondemand_labels_host(const float* f, const int64_t dims[3], const msc_integ_params* params,
                             const msc_triage_params* triage, int32_t* labels_asc, int32_t* labels_dsc) {
  return labels_host_impl(f, dims, params, triage, labels_asc, labels_dsc);
}

}  // extern "C"
