// extern "C" entry points of libmsc_gpu.so (declared in include/msc_gpu.h).
//
// Host-side orchestration of the .grad pipeline: argument checks, per-call scratch
// (two status words), kernel launches on the caller's stream, the ascending-manifold
// pass loop and error reporting.  Status codes only; nothing throws across the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <map>
#include <cstdlib>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "msc_device.cuh"
#include "../../include/msc_gpu.h"

namespace {

thread_local std::string g_last_error;
thread_local int g_last_passes = 0;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? MSC_ERR_OOM : MSC_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define MSC_CUDA(call, what)                  \
  do {                                        \
    cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

int num_sms() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 148;
  return n;
}

// Builds the mesh description, including the pair-code maps that reproduce the
// reference encoder when an axis has a single vertex
// (Compress6NeighborOffsetToByte, gi_topological_regular_grid.h:1182-1192: the
// first axis whose stride equals the offset wins).  Returns false on bad dims.
bool make_dims(int nd, const int64_t* dims, msc::GradDims* D) {
  if (!dims) return false;
  int64_t v[3] = {dims[0], dims[1], nd == 3 ? dims[2] : 1};
  for (int a = 0; a < 3; a++)
    if (v[a] < 1 || v[a] > (int64_t)1 << 30) return false;
  msc::GradDims d{};
  for (int a = 0; a < 3; a++) {
    d.v[a] = v[a];
    d.d[a] = 2 * v[a] - 1;
  }
  d.cs[0] = 1;
  d.cs[1] = d.d[0];
  d.cs[2] = d.d[0] * d.d[1];
  d.ncells = d.d[0] * d.d[1] * d.d[2];
  if (d.ncells / d.d[2] != d.d[0] * d.d[1]) return false;  // overflow
  uint32_t enc = 0, dec = 0;
  for (int c = 0; c < 6; c++) {
    const int a = c >> 1, s = c & 1;
    int e = c, t = c;
    if (nd == 3) {
      for (int b = 0; b < 3; b++)
        if (d.cs[b] == d.cs[a]) { e = 2 * b + s; break; }
      for (int b = 2; b >= 0; b--)
        if (d.cs[b] == d.cs[a]) { t = 2 * b + s; break; }
    }
    enc |= (uint32_t)e << (3 * c);
    dec |= (uint32_t)t << (3 * c);
  }
  d.enc_map = enc;
  d.dec_map = dec;
  *D = d;
  return true;
}

}  // namespace

namespace msc {
bool make_grad_dims(int nd, const int64_t* dims, GradDims* D) { return make_dims(nd, dims, D); }
}  // namespace msc

namespace {

struct Scratch {
  int* words = nullptr;  // [0] error bits, [1] changed flag
  cudaStream_t stream = nullptr;
  ~Scratch() {
    if (words) cudaFreeAsync(words, stream);
  }
};

int alloc_scratch(Scratch& s, cudaStream_t stream) {
  s.stream = stream;
  MSC_CUDA(msc::scratch_alloc((void**)&s.words, 2 * sizeof(int), stream), "scratch alloc(status words)");
  MSC_CUDA(cudaMemsetAsync(s.words, 0, 2 * sizeof(int), stream), "cudaMemsetAsync(status words)");
  return MSC_OK;
}

int check_errors(const Scratch& s, cudaStream_t stream) {
  int err = 0;
  MSC_CUDA(cudaMemcpyAsync(&err, s.words, sizeof(int), cudaMemcpyDeviceToHost, stream), "read status");
  MSC_CUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  if (err & msc::kErrNaN) return fail(MSC_ERR_NAN_INPUT, "input contains NaN");
  if (err & msc::kErrLocalQueue) return fail(MSC_ERR_QUEUE_OVERFLOW, "ldir tile queue overflow");
  if (err & msc::kErrPassLimit) return fail(MSC_ERR_ITER_LIMIT, "ldir closure did not converge");
  return MSC_OK;
}

int pairs_impl(int nd, const float* f, const int64_t* dims, uint8_t* g, cudaStream_t stream, Scratch& s) {
  msc::GradDims D;
  if (!make_dims(nd, dims, &D)) return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  if (!f || !g) return fail(MSC_ERR_NULL_POINTER, "null buffer");
  MSC_CUDA(msc::launch_lstar(nd, f, g, D, s.words, num_sms(), stream), "lower-star kernel launch");
  return MSC_OK;
}

// Multi-pass form: tile passes until no pass changes a cell near a tile border.
// `launches` counts kernel launches.
int ldir_passes(int nd, uint8_t* g, const msc::GradDims& D, cudaStream_t stream, Scratch& s, int* launches) {
  const int64_t ntiles = msc::ldir_num_tiles(nd, D);
  // one "reopened" byte per tile, double-buffered between passes
  uint8_t* dirty = nullptr;
  MSC_CUDA(msc::scratch_alloc((void**)&dirty, (size_t)(2 * ntiles), stream), "scratch alloc(tile flags)");
  struct Free {
    uint8_t* p;
    cudaStream_t st;
    ~Free() { cudaFreeAsync(p, st); }
  } free_dirty{dirty, stream};
  // a path that needs another pass crosses a tile border, so the closure completes
  // within (number of tiles + 1) passes
  const int64_t limit = ntiles + 2;
  const int sms = num_sms();
  int passes = 0;
  const uint8_t* din = nullptr;
  uint8_t* dout = dirty;
  while (true) {
    MSC_CUDA(cudaMemsetAsync(s.words + 1, 0, sizeof(int), stream), "reset changed flag");
    MSC_CUDA(cudaMemsetAsync(dout, 0, (size_t)ntiles, stream), "reset tile flags");
    MSC_CUDA(msc::launch_ldir_pass(nd, g, D, din, dout, s.words + 1, s.words, sms, stream), "ldir kernel launch");
    passes++;
    int changed = 0;
    MSC_CUDA(cudaMemcpyAsync(&changed, s.words + 1, sizeof(int), cudaMemcpyDeviceToHost, stream), "read changed");
    MSC_CUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    if (!changed) break;
    if (passes >= limit) return fail(MSC_ERR_ITER_LIMIT, "ldir closure did not converge");
    din = dout;
    dout = (dout == dirty) ? dirty + ntiles : dirty;
  }
  *launches += passes;
  return MSC_OK;
}

// Single-pass form: one tile pass that records the halo cells every tile lowered, a
// check of those records against the owners' cells, and global walks from the items
// the check lowered.  Should a frontier queue overflow, the multi-pass form finishes the
// closure from wherever it stands (the closure is monotone, so any intermediate
// state is a valid start).
// Frontier queue capacity for `ntiles` tiles; MSC_LDIR_QUEUE_CAP lowers it (tests of
// the multi-pass fallback).
int frontier_cap(int64_t ntiles) {
  int cap = (int)std::min<int64_t>(std::max<int64_t>(ntiles * 256, 1 << 16), (int64_t)1 << 30);
  if (const char* e = std::getenv("MSC_LDIR_QUEUE_CAP")) {
    const long v = std::strtol(e, nullptr, 10);
    if (v > 0 && v < cap) cap = (int)v;
  }
  return cap;
}

int ldir_batch_impl(int nd, const msc::LdirBatch& B, cudaStream_t stream, Scratch& s, int* passes_out) {
  const int64_t ntiles = B.total_tiles;
  const int64_t box = msc::ldir_halo_bytes(nd);
  const int sms = num_sms();
  const int cap = frontier_cap(ntiles);
  uint8_t* saved = nullptr;
  int64_t* queues = nullptr;
  int* ctr = nullptr;  // [0] queue a [1] queue b [2] lock [3] frontier overflow / CAS limit
  MSC_CUDA(msc::scratch_alloc((void**)&saved, (size_t)(ntiles * box), stream), "scratch alloc(halo records)");
  struct FreeAll {
    void* p[3];
    cudaStream_t st;
    ~FreeAll() {
      for (void* q : p)
        if (q) cudaFreeAsync(q, st);
    }
  } fr{{saved, nullptr, nullptr}, stream};
  MSC_CUDA(msc::scratch_alloc((void**)&queues, (size_t)cap * 2 * sizeof(int64_t), stream), "scratch alloc(queues)");
  fr.p[1] = queues;
  MSC_CUDA(msc::scratch_alloc((void**)&ctr, 4 * sizeof(int), stream), "scratch alloc(counters)");
  fr.p[2] = ctr;
  MSC_CUDA(cudaMemsetAsync(ctr, 0, 4 * sizeof(int), stream), "cudaMemsetAsync(counters)");

  int launches = 0;
  MSC_CUDA(msc::launch_ldir_tile(nd, B, saved, s.words, sms, stream), "ldir tile kernel launch");
  MSC_CUDA(msc::launch_ldir_check(nd, B, saved, queues, ctr, cap, ctr + 2, ctr + 3, sms, stream),
           "ldir check kernel launch");
  launches += 2;
  int64_t* qa = queues;
  int64_t* qb = queues + cap;
  bool overflow = false;
  for (int round = 0;; round++) {
    int h[4];
    MSC_CUDA(cudaMemcpyAsync(h, ctr, 4 * sizeof(int), cudaMemcpyDeviceToHost, stream), "read counters");
    MSC_CUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    const int n = round % 2 == 0 ? h[0] : h[1];
    if (h[3] || n > cap) {
      overflow = true;
      break;
    }
    if (n == 0) break;
    if (round > 4096) return fail(MSC_ERR_ITER_LIMIT, "ldir frontier walk did not converge");
    int* n_out = round % 2 == 0 ? ctr + 1 : ctr;
    MSC_CUDA(cudaMemsetAsync(n_out, 0, sizeof(int), stream), "reset queue");
    MSC_CUDA(msc::launch_ldir_walk(nd, B, qa, n, qb, n_out, cap, ctr + 2, ctr + 3, sms, stream),
             "ldir walk kernel launch");
    launches++;
    std::swap(qa, qb);
  }
  if (overflow) {
    for (int i = 0; i < B.n; i++)
      if (int rc = ldir_passes(nd, B.v[i].g, B.v[i].D, stream, s, &launches)) return rc;
  }
  if (passes_out) *passes_out = launches;
  g_last_passes = launches;
  return MSC_OK;
}

int ldir_impl(int nd, uint8_t* g, const int64_t* dims, cudaStream_t stream, Scratch& s, int* passes_out) {
  msc::GradDims D;
  if (!make_dims(nd, dims, &D)) return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  if (!g) return fail(MSC_ERR_NULL_POINTER, "null buffer");
  msc::LdirBatch B;
  MSC_CUDA(msc::make_ldir_batch(nd, 1, &g, &D, &B), "ldir batch");
  return ldir_batch_impl(nd, B, stream, s, passes_out);
}

int validate(int nd, const int64_t* dims, const void* a, const void* b) {
  msc::GradDims D;
  if (!make_dims(nd, dims, &D)) return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  if (!a || !b) return fail(MSC_ERR_NULL_POINTER, "null buffer");
  return MSC_OK;
}

int grad_impl(int nd, const float* f, const int64_t* dims, uint8_t* g, cudaStream_t stream) {
  if (int rc = validate(nd, dims, f, g)) return rc;
  Scratch s;
  int rc = alloc_scratch(s, stream);
  if (rc) return rc;
  rc = pairs_impl(nd, f, dims, g, stream, s);
  if (rc) return rc;
  rc = ldir_impl(nd, g, dims, stream, s, nullptr);
  if (rc) return rc;
  return check_errors(s, stream);
}

// The accurate 3-manifold .grad of ondemandaccurate from a base .grad and the final
// labels (msc_conforming_grad_3d).
int conform_impl(const float* f, const int32_t* asc, const int32_t* dsc, const int64_t* dims, uint8_t* g,
                 uint8_t* restrict_out, int64_t* touched_out, cudaStream_t stream) {
  msc::GradDims D;
  if (!make_dims(3, dims, &D)) return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  if (!f || !g) return fail(MSC_ERR_NULL_POINTER, "null buffer");
  Scratch s;
  if (int rc = alloc_scratch(s, stream)) return rc;
  uint8_t* rl = restrict_out;
  unsigned long long* touched = nullptr;
  struct Free {
    void* a;
    void* b;
    cudaStream_t st;
    ~Free() {
      if (a) cudaFreeAsync(a, st);
      if (b) cudaFreeAsync(b, st);
    }
  } fr{nullptr, nullptr, stream};
  if (!rl) {
    MSC_CUDA(msc::scratch_alloc((void**)&rl, (size_t)D.ncells, stream), "scratch alloc(restriction labels)");
    fr.a = rl;
  }
  MSC_CUDA(msc::scratch_alloc((void**)&touched, sizeof(unsigned long long), stream), "scratch alloc(counter)");
  fr.b = touched;
  MSC_CUDA(cudaMemsetAsync(touched, 0, sizeof(unsigned long long), stream), "cudaMemsetAsync");
  const int sms = num_sms();
  MSC_CUDA(msc::launch_restriction_labels(asc, dsc, f, D, rl, sms, stream), "restriction labels");
  MSC_CUDA(msc::launch_conform(f, rl, g, D, touched, sms, stream), "conforming re-pairing");
  if (int rc = ldir_impl(3, g, dims, stream, s, nullptr)) return rc;
  if (touched_out) {
    unsigned long long h = 0;
    MSC_CUDA(cudaMemcpyAsync(&h, touched, sizeof(h), cudaMemcpyDeviceToHost, stream), "read counter");
    MSC_CUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    *touched_out = (int64_t)h;
  }
  return check_errors(s, stream);
}

// Per-thread device staging for the host-buffer entries: grown on demand and kept
// between calls so repeated calls do not pay for allocation.
struct HostStaging {
  int dev = -1;
  float* f = nullptr;
  size_t fcap = 0;
  uint8_t* g = nullptr;
  size_t gcap = 0;
  cudaStream_t stream = nullptr;
};
thread_local HostStaging t_stage;

int ensure_staging(size_t fbytes, size_t gbytes) {
  int dev = 0;
  MSC_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  HostStaging& h = t_stage;
  if (h.dev != dev) {  // a different device: start over (old buffers belong to the old device)
    h = HostStaging{};
    h.dev = dev;
  }
  if (!h.stream) MSC_CUDA(cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking), "cudaStreamCreate");
  if (h.fcap < fbytes) {
    if (h.f) cudaFree(h.f);
    h.f = nullptr;
    h.fcap = 0;
    MSC_CUDA(cudaMalloc((void**)&h.f, fbytes), "cudaMalloc(f staging)");
    h.fcap = fbytes;
  }
  if (h.gcap < gbytes) {
    if (h.g) cudaFree(h.g);
    h.g = nullptr;
    h.gcap = 0;
    MSC_CUDA(cudaMalloc((void**)&h.g, gbytes), "cudaMalloc(grad staging)");
    h.gcap = gbytes;
  }
  return MSC_OK;
}

int host_impl(int nd, const float* fh, const int64_t* dims, uint8_t* gh) {
  msc::GradDims D;
  if (!make_dims(nd, dims, &D)) return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  if (!fh || !gh) return fail(MSC_ERR_NULL_POINTER, "null buffer");
  const size_t nv = (size_t)(D.v[0] * D.v[1] * D.v[2]);
  if (int rc = ensure_staging(nv * sizeof(float), (size_t)D.ncells)) return rc;
  HostStaging& h = t_stage;
  MSC_CUDA(cudaMemcpyAsync(h.f, fh, nv * sizeof(float), cudaMemcpyHostToDevice, h.stream), "copy f to device");
  if (int rc = grad_impl(nd, h.f, dims, h.g, h.stream)) return rc;
  MSC_CUDA(cudaMemcpyAsync(gh, h.g, (size_t)D.ncells, cudaMemcpyDeviceToHost, h.stream), "copy grad to host");
  MSC_CUDA(cudaStreamSynchronize(h.stream), "cudaStreamSynchronize");
  return MSC_OK;
}

// ---- batches of up to kMaxBatch volumes as one CUDA graph -------------------------------------
//
// The .grad of a batch is one graph: K1 over all volumes, the ldir tile pass, the halo
// check and kGraphRounds frontier-walk rounds whose queue lengths stay on the device.
// After a replay the host reads the counters once; a frontier left over after the
// captured rounds is walked on, an overflow falls back to tile passes.  The launch
// shapes (K1 blocks per SM, ldir tiles per SM) are picked by timing the candidates on
// the first batch of a size class; the instantiated graph is kept and replayed while
// the same buffers come back.

constexpr int kGraphRounds = 3;
constexpr int kGraphKernels = 3 + kGraphRounds;  // K1, tile, check, walk rounds

struct BatchGraph {
  int dev = -1;
  std::vector<const float*> f;
  std::vector<uint8_t*> g;
  std::vector<int64_t> dims;
  int bps = 64, cps = 4;
  cudaGraphExec_t exec = nullptr;
  uint8_t* saved = nullptr;
  int64_t* queues = nullptr;
  int* ctr = nullptr;    // [0] [1] queue lengths, [2] lock, [3] overflow / CAS limit
  int* words = nullptr;  // kernel status words
  int cap = 0;
  void release() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    for (void* q : {(void*)saved, (void*)queues, (void*)ctr, (void*)words})
      if (q) cudaFree(q);
    saved = nullptr;
    queues = nullptr;
    ctr = nullptr;
    words = nullptr;
  }
  ~BatchGraph() { release(); }
};
thread_local BatchGraph t_bgraph;
std::mutex g_tune_mu;
std::map<int, std::pair<int, int>> g_tuned;  // size class -> (K1 blocks per SM, ldir tiles per SM)

int capture_batch_graph(BatchGraph& G, const msc::LstarBatch& LB, const msc::LdirBatch& B, int bps, int cps,
                        cudaGraphExec_t* out) {
  const int sms = num_sms();
  cudaStream_t cs = nullptr;
  MSC_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate");
  struct Destroy {
    cudaStream_t s;
    ~Destroy() { cudaStreamDestroy(s); }
  } ds{cs};
  const long long counted = msc::launches_so_far();  // captured launches do not run now
  MSC_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
  cudaError_t e = cudaMemsetAsync(G.words, 0, 2 * sizeof(int), cs);
  if (e == cudaSuccess) e = cudaMemsetAsync(G.ctr, 0, 4 * sizeof(int), cs);
  if (e == cudaSuccess) e = msc::launch_lstar_batch(LB, G.words, sms, cs, bps);
  if (e == cudaSuccess) e = msc::launch_ldir_tile(3, B, G.saved, G.words, sms, cs, cps);
  if (e == cudaSuccess) e = msc::launch_ldir_check(3, B, G.saved, G.queues, G.ctr, G.cap, G.ctr + 2, G.ctr + 3, sms, cs);
  for (int r = 0; r < kGraphRounds && e == cudaSuccess; r++) {
    int* n_in = G.ctr + (r % 2);
    int* n_out = G.ctr + ((r + 1) % 2);
    e = cudaMemsetAsync(n_out, 0, sizeof(int), cs);
    if (e == cudaSuccess)
      e = msc::launch_ldir_walk_dev(B, G.queues + (size_t)(r % 2) * G.cap, n_in,
                                    G.queues + (size_t)((r + 1) % 2) * G.cap, n_out, G.cap, G.ctr + 2, G.ctr + 3, sms,
                                    cs);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(cs, &graph);
  msc::add_launches(counted - msc::launches_so_far());
  if (e == cudaSuccess) e = ec;
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  MSC_CUDA(e, "batch graph capture");
  return MSC_OK;
}

// Finishes what the captured rounds left: more walk rounds, or tile passes on overflow.
int finish_batch(BatchGraph& G, const msc::LdirBatch& B, cudaStream_t stream, int* launches) {
  const int sms = num_sms();
  int h[4];
  MSC_CUDA(cudaMemcpyAsync(h, G.ctr, 4 * sizeof(int), cudaMemcpyDeviceToHost, stream), "read counters");
  MSC_CUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  int cur = kGraphRounds % 2;
  int n = h[cur];
  bool overflow = h[3] != 0 || h[0] > G.cap || h[1] > G.cap;
  for (int round = 0; !overflow && n > 0; round++) {
    if (round > 4096) return fail(MSC_ERR_ITER_LIMIT, "ldir frontier walk did not converge");
    int* n_out = G.ctr + (1 - cur);
    MSC_CUDA(cudaMemsetAsync(n_out, 0, sizeof(int), stream), "reset queue");
    MSC_CUDA(msc::launch_ldir_walk(3, B, G.queues + (size_t)cur * G.cap, n, G.queues + (size_t)(1 - cur) * G.cap, n_out,
                                   G.cap, G.ctr + 2, G.ctr + 3, sms, stream),
             "ldir walk kernel launch");
    (*launches)++;
    MSC_CUDA(cudaMemcpyAsync(h, G.ctr, 4 * sizeof(int), cudaMemcpyDeviceToHost, stream), "read counters");
    MSC_CUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    cur = 1 - cur;
    n = h[cur];
    overflow = h[3] != 0 || n > G.cap;
  }
  if (overflow) {
    Scratch s;
    if (int rc = alloc_scratch(s, stream)) return rc;
    for (int i = 0; i < B.n; i++)
      if (int rc = ldir_passes(3, B.v[i].g, B.v[i].D, stream, s, launches)) return rc;
    if (int rc = check_errors(s, stream)) return rc;
  }
  return MSC_OK;
}

int grad_batch_graph_impl(int n, const float* const* f, const int64_t* dims, uint8_t* const* g,
                          const std::vector<msc::GradDims>& D, cudaStream_t stream) {
  int dev = 0;
  MSC_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  BatchGraph& G = t_bgraph;
  msc::LstarBatch LB;
  msc::LdirBatch B;
  MSC_CUDA(msc::make_lstar_batch(n, f, g, D.data(), &LB), "lower-star batch (plane too large)");
  MSC_CUDA(msc::make_ldir_batch(3, n, g, D.data(), &B), "ldir batch");
  const int cap = frontier_cap(B.total_tiles);
  const bool same = G.exec && G.dev == dev && G.cap == cap && (int)G.f.size() == n &&
                    std::equal(G.f.begin(), G.f.end(), f) && std::equal(G.g.begin(), G.g.end(), g) &&
                    std::equal(G.dims.begin(), G.dims.end(), dims);
  if (!same) {
    G.release();
    G.dev = dev;
    G.f.assign(f, f + n);
    G.g.assign(g, g + n);
    G.dims.assign(dims, dims + 3 * n);
    G.cap = cap;
    MSC_CUDA(cudaMalloc((void**)&G.saved, (size_t)B.total_tiles * msc::ldir_halo_bytes(3)), "cudaMalloc(saved halos)");
    MSC_CUDA(cudaMalloc((void**)&G.queues, (size_t)G.cap * 2 * sizeof(int64_t)), "cudaMalloc(queues)");
    MSC_CUDA(cudaMalloc((void**)&G.ctr, 4 * sizeof(int)), "cudaMalloc(counters)");
    MSC_CUDA(cudaMalloc((void**)&G.words, 2 * sizeof(int)), "cudaMalloc(status)");
    // launch shapes: tuned once per size class (log2 of the tile count)
    int cls = 0;
    for (int64_t t = B.total_tiles; t > 1; t >>= 1) cls++;
    std::pair<int, int> best{64, 4};
    bool tuned = false;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tuned.find(cls);
      if (it != g_tuned.end()) {
        best = it->second;
        tuned = true;
      }
    }
    if (!tuned && B.total_tiles >= 256) {
      float best_ms = 1e30f;
      cudaEvent_t e0, e1;
      MSC_CUDA(cudaEventCreate(&e0), "cudaEventCreate");
      MSC_CUDA(cudaEventCreate(&e1), "cudaEventCreate");
      for (int bps : {32, 64, 128})
        for (int cps : {2, 4}) {
          cudaGraphExec_t ex = nullptr;
          if (int rc = capture_batch_graph(G, LB, B, bps, cps, &ex)) return rc;
          cudaGraphLaunch(ex, stream);
          cudaEventRecord(e0, stream);
          cudaGraphLaunch(ex, stream);
          cudaEventRecord(e1, stream);
          msc::add_launches(2 * kGraphKernels);
          MSC_CUDA(cudaEventSynchronize(e1), "autotune");
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          cudaGraphExecDestroy(ex);
          if (ms < best_ms) {
            best_ms = ms;
            best = {bps, cps};
          }
        }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tuned[cls] = best;
    }
    G.bps = best.first;
    G.cps = best.second;
    if (int rc = capture_batch_graph(G, LB, B, G.bps, G.cps, &G.exec)) return rc;
  }
  MSC_CUDA(cudaGraphLaunch(G.exec, stream), "cudaGraphLaunch");
  msc::add_launches(kGraphKernels);
  int launches = kGraphKernels;
  if (int rc = finish_batch(G, B, stream, &launches)) return rc;
  g_last_passes = launches;
  int err = 0;
  MSC_CUDA(cudaMemcpyAsync(&err, G.words, sizeof(int), cudaMemcpyDeviceToHost, stream), "read status");
  MSC_CUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  if (err & msc::kErrNaN) return fail(MSC_ERR_NAN_INPUT, "input contains NaN");
  if (err & msc::kErrLocalQueue) return fail(MSC_ERR_QUEUE_OVERFLOW, "ldir tile queue overflow");
  return MSC_OK;
}

// Many 3D volumes: one K1 launch and one ldir tile / check / walk sequence per chunk
// of up to kMaxBatch volumes.
int grad_batch_impl(int n, const float* const* f, const int64_t* dims, uint8_t* const* g, cudaStream_t stream) {
  if (n < 0) return fail(MSC_ERR_BAD_DIMS, "negative batch size");
  if (n == 0) return MSC_OK;
  if (!f || !dims || !g) return fail(MSC_ERR_NULL_POINTER, "null argument");
  std::vector<msc::GradDims> D(n);
  for (int i = 0; i < n; i++) {
    if (!make_dims(3, dims + 3 * i, &D[i])) return fail(MSC_ERR_BAD_DIMS, "invalid dims of volume " + std::to_string(i));
    if (!f[i] || !g[i]) return fail(MSC_ERR_NULL_POINTER, "null buffer of volume " + std::to_string(i));
  }
  if (n <= msc::kMaxBatch) return grad_batch_graph_impl(n, f, dims, g, D, stream);
  Scratch s;
  if (int rc = alloc_scratch(s, stream)) return rc;
  const int sms = num_sms();
  int launches = 0;
  for (int i0 = 0; i0 < n; i0 += msc::kMaxBatch) {
    const int m = std::min(n - i0, msc::kMaxBatch);
    msc::LstarBatch LB;
    MSC_CUDA(msc::make_lstar_batch(m, f + i0, g + i0, D.data() + i0, &LB), "lower-star batch (plane too large)");
    MSC_CUDA(msc::launch_lstar_batch(LB, s.words, sms, stream), "lower-star batch kernel launch");
    msc::LdirBatch B;
    MSC_CUDA(msc::make_ldir_batch(3, m, g + i0, D.data() + i0, &B), "ldir batch");
    int l = 0;
    if (int rc = ldir_batch_impl(3, B, stream, s, &l)) return rc;
    launches += 1 + l;
  }
  g_last_passes = launches;
  return check_errors(s, stream);
}

}  // namespace

namespace msc {
// Records the calling thread's error text for msc_last_error_string().
int set_last_error(int code, const char* msg) { return fail(code, msg); }

// A 512^3 labeling call takes ~18 GB of scratch per direction, a .grad call ~0.4 GB;
// mapping that afresh on every call (the default pool hands memory back at every
// synchronisation) cost 0.09 s of a 0.72 s labeling call.
std::mutex g_pool_mu;
std::map<int, cudaMemPool_t> g_pools;

cudaError_t scratch_pool(cudaMemPool_t* out) {
  int dev = 0;
  if (cudaError_t e = cudaGetDevice(&dev)) return e;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  auto it = g_pools.find(dev);
  if (it != g_pools.end()) {
    *out = it->second;
    return cudaSuccess;
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  if (cudaError_t e = cudaMemPoolCreate(&pool, &props)) return e;
  uint64_t keep = ~0ull;
  if (cudaError_t e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep)) return e;
  g_pools[dev] = pool;
  *out = pool;
  return cudaSuccess;
}

cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t stream) {
  cudaMemPool_t pool = nullptr;
  if (cudaError_t e = scratch_pool(&pool)) return e;
  return cudaMallocFromPoolAsync(p, bytes, pool, stream);
}

std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void add_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace msc

extern "C" {

int msc_version(void) { return 100; }

const char* msc_last_error_string(void) { return g_last_error.c_str(); }

int msc_last_ldir_passes(void) { return g_last_passes; }

void msc_trim_scratch(void) {
  std::lock_guard<std::mutex> lk(msc::g_pool_mu);
  for (auto& kv : msc::g_pools) cudaMemPoolTrimTo(kv.second, 0);
}

int64_t msc_kernel_launches(void) { return (int64_t)msc::g_launches.load(std::memory_order_relaxed); }

int64_t msc_num_cells_3d(const int64_t dims[3]) {
  msc::GradDims D;
  return make_dims(3, dims, &D) ? D.ncells : -1;
}

int64_t msc_num_cells_2d(const int64_t dims[2]) {
  msc::GradDims D;
  return make_dims(2, dims, &D) ? D.ncells : -1;
}

int msc_lower_star_grad_3d(const float* f, const int64_t dims[3], uint8_t* g, msc_stream_t stream) {
  return grad_impl(3, f, dims, g, (cudaStream_t)stream);
}

int msc_lower_star_grad_batch_3d(int n, const float* const* f, const int64_t* dims, uint8_t* const* grad,
                                 msc_stream_t stream) {
  return grad_batch_impl(n, f, dims, grad, (cudaStream_t)stream);
}

int msc_lower_star_grad_2d(const float* f, const int64_t dims[2], uint8_t* g, msc_stream_t stream) {
  return grad_impl(2, f, dims, g, (cudaStream_t)stream);
}

int msc_lower_star_pairs_3d(const float* f, const int64_t dims[3], uint8_t* g, msc_stream_t stream) {
  if (int rc = validate(3, dims, f, g)) return rc;
  Scratch s;
  int rc = alloc_scratch(s, (cudaStream_t)stream);
  if (!rc) rc = pairs_impl(3, f, dims, g, (cudaStream_t)stream, s);
  if (!rc) rc = check_errors(s, (cudaStream_t)stream);
  return rc;
}

int msc_lower_star_pairs_2d(const float* f, const int64_t dims[2], uint8_t* g, msc_stream_t stream) {
  if (int rc = validate(2, dims, f, g)) return rc;
  Scratch s;
  int rc = alloc_scratch(s, (cudaStream_t)stream);
  if (!rc) rc = pairs_impl(2, f, dims, g, (cudaStream_t)stream, s);
  if (!rc) rc = check_errors(s, (cudaStream_t)stream);
  return rc;
}

int msc_ascending_manifold_dims_3d(uint8_t* g, const int64_t dims[3], msc_stream_t stream, int* passes_out) {
  if (int rc = validate(3, dims, g, g)) return rc;
  Scratch s;
  int rc = alloc_scratch(s, (cudaStream_t)stream);
  if (!rc) rc = ldir_impl(3, g, dims, (cudaStream_t)stream, s, passes_out);
  if (!rc) rc = check_errors(s, (cudaStream_t)stream);
  return rc;
}

int msc_ascending_manifold_dims_2d(uint8_t* g, const int64_t dims[2], msc_stream_t stream, int* passes_out) {
  if (int rc = validate(2, dims, g, g)) return rc;
  Scratch s;
  int rc = alloc_scratch(s, (cudaStream_t)stream);
  if (!rc) rc = ldir_impl(2, g, dims, (cudaStream_t)stream, s, passes_out);
  if (!rc) rc = check_errors(s, (cudaStream_t)stream);
  return rc;
}

int msc_central_diff_grad_3d(const float* f, const int64_t dims[3], float* g, int layout, msc_stream_t stream) {
  if (int rc = validate(3, dims, f, g)) return rc;
  if (layout != 0 && layout != 1) return fail(MSC_ERR_BAD_DIMS, "layout must be 0 (xyz) or 1 (xyzw)");
  msc::GradDims D;
  make_dims(3, dims, &D);
  MSC_CUDA(msc::launch_central_diff(3, layout, f, g, D, num_sms(), (cudaStream_t)stream), "gradient kernel launch");
  return MSC_OK;
}

int msc_central_diff_grad_2d(const float* f, const int64_t dims[2], float* g, int layout, msc_stream_t stream) {
  if (int rc = validate(2, dims, f, g)) return rc;
  if (layout != 0 && layout != 1) return fail(MSC_ERR_BAD_DIMS, "layout must be 0 (xy) or 1 (xy, 8-byte aligned pairs)");
  msc::GradDims D;
  make_dims(2, dims, &D);
  MSC_CUDA(msc::launch_central_diff(2, layout, f, g, D, num_sms(), (cudaStream_t)stream), "gradient kernel launch");
  return MSC_OK;
}

int msc_central_diff_grad_3d_f64(const float* f, const int64_t dims[3], double* g, msc_stream_t stream) {
  if (int rc = validate(3, dims, f, g)) return rc;
  msc::GradDims D;
  make_dims(3, dims, &D);
  MSC_CUDA(msc::launch_central_diff(3, 2, f, g, D, num_sms(), (cudaStream_t)stream), "gradient kernel launch");
  return MSC_OK;
}

int msc_central_diff_grad_2d_f64(const float* f, const int64_t dims[2], double* g, msc_stream_t stream) {
  if (int rc = validate(2, dims, f, g)) return rc;
  msc::GradDims D;
  make_dims(2, dims, &D);
  MSC_CUDA(msc::launch_central_diff(2, 2, f, g, D, num_sms(), (cudaStream_t)stream), "gradient kernel launch");
  return MSC_OK;
}

int msc_conforming_grad_3d(const float* f, const int32_t* labels_asc, const int32_t* labels_dsc, const int64_t dims[3],
                           uint8_t* grad, uint8_t* restriction_out, int64_t* touched_out, msc_stream_t stream) {
  return conform_impl(f, labels_asc, labels_dsc, dims, grad, restriction_out, touched_out, (cudaStream_t)stream);
}

int msc_steepest_lstar_host(const float* f_host, const int64_t dims[3], uint8_t* grad_host) {
  return host_impl(3, f_host, dims, grad_host);
}

int msc_lower_star_grad_2d_host(const float* f_host, const int64_t dims[2], uint8_t* grad_host) {
  return host_impl(2, f_host, dims, grad_host);
}

}  // extern "C"
