// The saddle streamline digitizers of ondemandaccurate's needASC1 / needDSC1 modes
// (ondemandaccurate.cxx:254-505, gi_numeric_streamline_integrator.h:525-1080) on the
// device: the parallel form of saddle_core.cuh as kernels.
//
// Per direction:
//   1. the critical saddles (2-cells ascending, 1-cells descending) with their order key
//      (value of the highest vertex, negated descending; then the cell id) packed into
//      64 bits and radix-sorted: the one-thread order is the descending sort;
//   2. each saddle's seed cells (a thread per saddle); items numbered by a scan: a
//      saddle's streamlines, then its own write;
//   3. every streamline integrated without labels twice, counting its voxel steps and
//      then recording them at scanned offsets (a thread per streamline, FP64);
//   4. rounds: claims = the labels present before (key 0), then each saddle's own write
//      and every streamline's live writes as atomicMin of their keys, against the
//      previous round's claims; a round that changes no claim ends the loop;
//   5. the cells with a claim take the direction's label.
// One thread per streamline, records of 136 bytes per voxel step: a first form whose
// cost is the label-free records (3.4-4.3x the voxel steps the one-thread run keeps on
// k^-3 fields); compact records and lazy speculation are its next steps.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "msc_device.cuh"
#include "msc_gpu.h"
#include "saddle_core.cuh"

namespace msc {
namespace {

using namespace sl;

constexpr int kThreads = 256;
constexpr int kMaxRounds = 4096;

enum : int { kLineErrOverflow = 1 };

int fail(int code, const std::string& m) { return set_last_error(code, m.c_str()); }
#define SCUDA(call, what)                                                                          \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return fail(e_ == cudaErrorMemoryAllocation ? MSC_ERR_OOM : MSC_ERR_CUDA,                   \
                  std::string(what) + ": " + cudaGetErrorString(e_));                              \
  } while (0)

struct Pool {
  std::vector<void*> p;
  cudaStream_t st;
  ~Pool() {
    for (void* q : p) cudaFreeAsync(q, st);
  }
  template <class T>
  cudaError_t get(T** out, size_t n) {
    void* q = nullptr;
    cudaError_t e = scratch_alloc(&q, n * sizeof(T) ? n * sizeof(T) : 16, st);
    if (e == cudaSuccess) p.push_back(q);
    *out = static_cast<T*>(q);
    return e;
  }
};

unsigned grid_for(int64_t n) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t b = (n + kThreads - 1) / kThreads, cap = (int64_t)sms * 8;
  return (unsigned)(b < 1 ? 1 : (b < cap ? b : cap));
}

// order-preserving bits of a float (no NaN: the .grad path rejects them); -0 and +0
// compare equal, as in the one-thread sort, and leave the order to the cell id
__device__ __forceinline__ uint32_t ordered_bits(float v) {
  if (v == 0.0f) v = 0.0f;
  const uint32_t u = __float_as_uint(v);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ bool vertex_greater(const float* f, int64_t a, int64_t b) {
  const float fa = f[a], fb = f[b];
  if (fa > fb) return true;
  if (fb > fa) return false;
  return a > b;
}

// 1. the critical saddles of dimension sdim: (ordered key << 32 | cell id), appended
// one atomic per warp (the loop is warp-uniform)
__global__ void saddle_keys_kernel(const uint8_t* __restrict__ grad, const float* __restrict__ f, Grid G, int dsc,
                                   uint64_t* __restrict__ keys, int64_t key_cap,
                                   unsigned long long* __restrict__ n_keys) {
  const int64_t nc = G.dX * G.dY * G.dZ;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t rounds = (nc + stride - 1) / stride;
  const int sdim = dsc ? 1 : 2;
  const unsigned lane = threadIdx.x & 31u;
  for (int64_t r = 0; r < rounds; r++) {
    const int64_t id = r * stride + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool take = false;
    uint64_t key = 0;
    if (id < nc && grad_critical(grad, id)) {
      int64_t k[3];
      cell_coords(G, id, k);
      if ((int)((k[0] & 1) + (k[1] & 1) + (k[2] & 1)) == sdim) {
        take = true;
        int64_t best = -1;
        for (int s = 0; s < 8; s++) {
          int64_t q[3];
          bool ok = true;
          for (int a = 0; a < 3; a++) {
            const int bit = (s >> a) & 1;
            if (!(k[a] & 1) && bit) ok = false;
            q[a] = (k[a] & 1) ? (bit ? k[a] + 1 : k[a] - 1) : k[a];
          }
          if (!ok) continue;
          const int64_t v = (q[0] >> 1) + (q[1] >> 1) * G.X + (q[2] >> 1) * G.X * G.Y;
          if (best < 0 || vertex_greater(f, v, best)) best = v;
        }
        const float val = f[best];
        key = ((uint64_t)ordered_bits(dsc ? -1 * val : val) << 32) | (uint64_t)(uint32_t)id;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) continue;
    unsigned long long base = 0;
    const int leader = __ffs(m) - 1;
    if ((int)lane == leader) base = atomicAdd(n_keys, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    const unsigned long long at = base + __popc(m & ((1u << lane) - 1u));
    if (take && at < (unsigned long long)key_cap) keys[at] = key;  // the host rejects a count above the cap
  }
}

// 2. seeds per saddle in the one-thread order (sorted ascending: saddle i is
// sorted[n - 1 - i]); items[i] = seeds + 1 (its streamlines and its own write)
__global__ void seed_count_kernel(const uint8_t* __restrict__ grad, Grid G, int dsc, const uint64_t* __restrict__ sorted,
                                  int64_t n, int64_t* __restrict__ items) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t sad = (int64_t)(uint32_t)sorted[n - 1 - i];
    int64_t seeds[kMaxSeeds];
    items[i] = saddle_seeds(G, grad, sad, dsc, seeds) + 1;
  }
}

// the streamlines (item number, seed cell) and the saddles' own writes (cell, item)
__global__ void seed_write_kernel(const uint8_t* __restrict__ grad, Grid G, int dsc, const uint64_t* __restrict__ sorted,
                                  int64_t n, const int64_t* __restrict__ item_base, uint32_t* __restrict__ line_item,
                                  int64_t* __restrict__ line_seed, int64_t* __restrict__ sad_cell,
                                  uint32_t* __restrict__ sad_item) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t sad = (int64_t)(uint32_t)sorted[n - 1 - i];
    int64_t seeds[kMaxSeeds];
    const int ns = saddle_seeds(G, grad, sad, dsc, seeds);
    const int64_t ib = item_base[i], lb = ib - i;  // streamlines before: items before minus saddles before
    for (int s = 0; s < ns; s++) {
      line_item[lb + s] = (uint32_t)(ib + s);
      line_seed[lb + s] = seeds[s];
    }
    sad_cell[i] = sad;
    sad_item[i] = (uint32_t)(ib + ns);
  }
}

__device__ __forceinline__ V3 seed_point(const Grid& G, int64_t cell) {
  int64_t k[3];
  cell_coords(G, cell, k);
  return {(double)k[0] * 0.5, (double)k[1] * 0.5, (double)k[2] * 0.5};
}

// 3. label-free streamlines: count their voxel steps (recs == nullptr) or record them
__global__ void trace_kernel(Field F, Params P, int dsc, const int64_t* __restrict__ line_seed, int64_t n_lines,
                             int64_t* __restrict__ n_steps, const int64_t* __restrict__ offsets,
                             StepRec* __restrict__ recs, int* __restrict__ err) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n_lines; j += (int64_t)gridDim.x * blockDim.x) {
    int64_t used = 0;
    const int64_t cap = recs ? n_steps[j] : INT64_MAX;
    StepRec* out = recs ? recs + offsets[j] : nullptr;
    const int r = trace_line(F, P, dsc, seed_point(F.g, line_seed[j]), [&](const StepRec& s) {
      if (used >= cap) return false;
      if (out) out[used] = s;
      used++;
      return true;
    });
    if (r < 0) atomicOr(err, kLineErrOverflow);
    if (!recs) n_steps[j] = used;
  }
}

__global__ void base_claims_kernel(const uint8_t* __restrict__ cells, int64_t nc, uint8_t target,
                                   unsigned long long* __restrict__ base) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x)
    base[c] = cells[c] == target ? 0ull : (unsigned long long)kNoClaim;
}

// 4. one round: the saddles' own writes and the streamlines' live writes against the
// previous round's claims
__global__ void saddle_claims_kernel(const int64_t* __restrict__ sad_cell, const uint32_t* __restrict__ sad_item,
                                     int64_t n, unsigned long long* __restrict__ next) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    atomicMin(next + sad_cell[i], (unsigned long long)event_key(sad_item[i], 0, 0));
}

__global__ void walk_kernel(Field F, Params P, int dsc, const uint32_t* __restrict__ line_item, int64_t n_lines,
                            const int64_t* __restrict__ n_steps, const int64_t* __restrict__ offsets,
                            const StepRec* __restrict__ recs, const unsigned long long* __restrict__ claim,
                            unsigned long long* __restrict__ next, unsigned long long* __restrict__ kept) {
  const int64_t nc = F.g.dX * F.g.dY * F.g.dZ;
  unsigned long long my_kept = 0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n_lines; j += (int64_t)gridDim.x * blockDim.x) {
    const StepRec* r = recs + offsets[j];
    my_kept += (unsigned long long)walk_line(
        F, P, dsc, line_item[j], [&](int t) -> const StepRec& { return r[t]; }, (int)n_steps[j],
        [&](int64_t c) -> uint64_t { return (uint64_t)c < (uint64_t)nc ? (uint64_t)claim[c] : 0ull; },
        [&](int64_t c, uint64_t key) {
          if ((uint64_t)c < (uint64_t)nc) atomicMin(next + c, (unsigned long long)key);
        });
  }
  if (my_kept) atomicAdd(kept, my_kept);
}

__global__ void changed_kernel(const unsigned long long* __restrict__ a, const unsigned long long* __restrict__ b,
                               int64_t nc, int* __restrict__ changed) {
  bool d = false;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x)
    d |= a[c] != b[c];
  if (__syncthreads_or(d) && threadIdx.x == 0) atomicOr(changed, 1);
}

// 5. the label of the direction on every claimed cell
__global__ void apply_kernel(const unsigned long long* __restrict__ claim, int64_t nc, uint8_t target,
                             uint8_t* __restrict__ cells) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x)
    if (claim[c] != (unsigned long long)kNoClaim) cells[c] = target;
}

int lines_direction(const Field& F, const Params& P, const uint8_t* grad, int dsc, uint8_t* cells, int64_t stats[4],
                    cudaStream_t st) {
  const Grid& G = F.g;
  const int64_t nc = G.dX * G.dY * G.dZ;
  const uint8_t target = dsc ? 5 : 4;
  Pool pool{{}, st};
  // 1. saddles, sorted
  uint64_t *keys, *sorted;
  unsigned long long* counters;  // [0] saddles [1] kept steps
  int* flags;                    // [0] changed [1] error
  SCUDA(pool.get(&counters, 2), "scratch alloc(counters)");
  SCUDA(pool.get(&flags, 2), "scratch alloc(flags)");
  SCUDA(cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), st), "cudaMemsetAsync");
  SCUDA(cudaMemsetAsync(flags, 0, 2 * sizeof(int), st), "cudaMemsetAsync");
  // at most one saddle per cell of its dimension: dX*dY*dZ / 2 bounds both kinds
  const int64_t key_cap = nc / 2 + 1;
  SCUDA(pool.get(&keys, (size_t)key_cap), "scratch alloc(saddle keys)");
  count_launch();
  saddle_keys_kernel<<<grid_for(nc), kThreads, 0, st>>>(grad, F.f, G, dsc, keys, key_cap, counters);
  SCUDA(cudaGetLastError(), "saddle_keys_kernel");
  unsigned long long h_n = 0;
  SCUDA(cudaMemcpyAsync(&h_n, counters, sizeof(h_n), cudaMemcpyDeviceToHost, st), "read saddle count");
  SCUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  const int64_t n = (int64_t)h_n;
  if (n == 0) return MSC_OK;
  if (n > key_cap) return fail(MSC_ERR_QUEUE_OVERFLOW, "more saddles than cells of their dimension");
  SCUDA(pool.get(&sorted, (size_t)n), "scratch alloc(sorted keys)");
  size_t tmp_bytes = 0, scan_bytes = 0;
  SCUDA(cub::DeviceRadixSort::SortKeys(nullptr, tmp_bytes, keys, sorted, n, 0, 64, st), "sort size");
  int64_t *items, *item_base;
  SCUDA(pool.get(&items, (size_t)n + 1), "scratch alloc(items)");
  SCUDA(pool.get(&item_base, (size_t)n + 1), "scratch alloc(items)");
  SCUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, items, item_base, n + 1, st), "scan size");
  void* tmp;
  SCUDA(pool.get(reinterpret_cast<uint8_t**>(&tmp), tmp_bytes > scan_bytes ? tmp_bytes : scan_bytes),
        "scratch alloc(sort)");
  SCUDA(cub::DeviceRadixSort::SortKeys(tmp, tmp_bytes, keys, sorted, n, 0, 64, st), "sort");
  // 2. seeds and items
  count_launch();
  seed_count_kernel<<<grid_for(n), kThreads, 0, st>>>(grad, G, dsc, sorted, n, items);
  SCUDA(cudaMemsetAsync(items + n, 0, sizeof(int64_t), st), "cudaMemsetAsync");
  size_t sb = scan_bytes;
  SCUDA(cub::DeviceScan::ExclusiveSum(tmp, sb, items, item_base, n + 1, st), "scan items");
  int64_t n_items = 0;
  SCUDA(cudaMemcpyAsync(&n_items, item_base + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "read item count");
  SCUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (n_items >= (int64_t)0xFFFFFFFEll) return fail(MSC_ERR_TOO_LARGE, "more than 2^32 - 2 streamlines and saddles");
  const int64_t n_lines = n_items - n;
  uint32_t *line_item, *sad_item;
  int64_t *line_seed, *sad_cell, *n_steps;
  SCUDA(pool.get(&line_item, (size_t)n_lines), "scratch alloc(lines)");
  SCUDA(pool.get(&line_seed, (size_t)n_lines), "scratch alloc(lines)");
  SCUDA(pool.get(&n_steps, (size_t)n_lines + 1), "scratch alloc(lines)");
  SCUDA(pool.get(&sad_cell, (size_t)n), "scratch alloc(saddles)");
  SCUDA(pool.get(&sad_item, (size_t)n), "scratch alloc(saddles)");
  count_launch();
  seed_write_kernel<<<grid_for(n), kThreads, 0, st>>>(grad, G, dsc, sorted, n, item_base, line_item, line_seed,
                                                       sad_cell, sad_item);
  // 3. label-free records: count, scan, record
  int64_t* offsets;
  SCUDA(pool.get(&offsets, (size_t)n_lines + 1), "scratch alloc(offsets)");
  if (n_lines > 0) {
    count_launch();
    trace_kernel<<<grid_for(n_lines), kThreads, 0, st>>>(F, P, dsc, line_seed, n_lines, n_steps, nullptr, nullptr,
                                                          flags + 1);
  }
  SCUDA(cudaMemsetAsync(n_steps + n_lines, 0, sizeof(int64_t), st), "cudaMemsetAsync");
  size_t ob = 0;
  SCUDA(cub::DeviceScan::ExclusiveSum(nullptr, ob, n_steps, offsets, n_lines + 1, st), "scan size");
  void* otmp;
  SCUDA(pool.get(reinterpret_cast<uint8_t**>(&otmp), ob), "scratch alloc(scan)");
  SCUDA(cub::DeviceScan::ExclusiveSum(otmp, ob, n_steps, offsets, n_lines + 1, st), "scan steps");
  int64_t n_recs = 0;
  int h_err = 0;
  SCUDA(cudaMemcpyAsync(&n_recs, offsets + n_lines, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "read steps");
  SCUDA(cudaMemcpyAsync(&h_err, flags + 1, sizeof(int), cudaMemcpyDeviceToHost, st), "read status");
  SCUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (h_err) return fail(MSC_ERR_QUEUE_OVERFLOW, "a voxel step entered more cells than a record holds");
  StepRec* recs;
  SCUDA(pool.get(&recs, (size_t)n_recs), "scratch alloc(step records)");
  if (n_lines > 0) {
    count_launch();
    trace_kernel<<<grid_for(n_lines), kThreads, 0, st>>>(F, P, dsc, line_seed, n_lines, n_steps, offsets, recs,
                                                          flags + 1);
  }
  // 4. rounds
  unsigned long long *base, *claim, *next;
  SCUDA(pool.get(&base, (size_t)nc), "scratch alloc(claims)");
  SCUDA(pool.get(&claim, (size_t)nc), "scratch alloc(claims)");
  SCUDA(pool.get(&next, (size_t)nc), "scratch alloc(claims)");
  count_launch();
  base_claims_kernel<<<grid_for(nc), kThreads, 0, st>>>(cells, nc, target, base);
  SCUDA(cudaMemcpyAsync(claim, base, (size_t)nc * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st),
        "copy claims");
  int rounds = 0;
  for (;;) {
    if (rounds == kMaxRounds) return fail(MSC_ERR_ITER_LIMIT, "saddle-line claims did not settle");
    SCUDA(cudaMemcpyAsync(next, base, (size_t)nc * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st),
          "copy claims");
    SCUDA(cudaMemsetAsync(flags, 0, sizeof(int), st), "cudaMemsetAsync");
    SCUDA(cudaMemsetAsync(counters + 1, 0, sizeof(unsigned long long), st), "cudaMemsetAsync");
    count_launch();
    saddle_claims_kernel<<<grid_for(n), kThreads, 0, st>>>(sad_cell, sad_item, n, next);
    if (n_lines > 0) {
      count_launch();
      walk_kernel<<<grid_for(n_lines), kThreads, 0, st>>>(F, P, dsc, line_item, n_lines, n_steps, offsets, recs, claim,
                                                         next, counters + 1);
    }
    count_launch();
    changed_kernel<<<grid_for(nc), kThreads, 0, st>>>(claim, next, nc, flags);
    SCUDA(cudaGetLastError(), "round launch");
    int changed = 0;
    SCUDA(cudaMemcpyAsync(&changed, flags, sizeof(int), cudaMemcpyDeviceToHost, st), "read round status");
    SCUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    rounds++;
    unsigned long long* t = claim;
    claim = next;
    next = t;
    if (!changed) break;
  }
  // 5. labels
  count_launch();
  apply_kernel<<<grid_for(nc), kThreads, 0, st>>>(claim, nc, target, cells);
  unsigned long long h_kept = 0;
  SCUDA(cudaMemcpyAsync(&h_kept, counters + 1, sizeof(h_kept), cudaMemcpyDeviceToHost, st), "read kept steps");
  SCUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  stats[0] += n_lines;
  stats[1] += n_recs;
  stats[2] += (int64_t)h_kept;
  if (rounds > stats[3]) stats[3] = rounds;
  return MSC_OK;
}

int saddle_lines_impl(const float* f, const uint8_t* grad, const uint32_t* zeroed, const int64_t* dims, int which,
                      const msc_integ_params* prm, uint8_t* cells, int64_t* stats_out, cudaStream_t st) {
  if (!dims || !prm) return fail(MSC_ERR_NULL_POINTER, "null argument");
  if (dims[0] < 2 || dims[1] < 2 || dims[2] < 2 || dims[0] > (1 << 20) || dims[1] > (1 << 20) || dims[2] > (1 << 20))
    return fail(MSC_ERR_BAD_DIMS, "invalid dims (2 or more vertices per axis)");
  const Grid G = make_grid(dims[0], dims[1], dims[2]);
  const int64_t nc = G.dX * G.dY * G.dZ;
  if (nc / G.dZ != G.dX * G.dY || nc >= ((int64_t)1 << 32)) return fail(MSC_ERR_TOO_LARGE, "2^32 or more cells");
  if (!f || !grad || !cells) return fail(MSC_ERR_NULL_POINTER, "null buffer");
  if ((which & ~3) || !which) return fail(MSC_ERR_BAD_DIMS, "which must be 1, 2 or 3");
  if (prm->iteration_limit < 0 || prm->iteration_limit >= (1 << 27))
    return fail(MSC_ERR_BAD_DIMS, "iteration_limit out of range");
  const Field F{f, zeroed, G};
  const Params P{prm->error_threshold, prm->gradient_threshold, (double)prm->max_step, prm->iteration_limit};
  int64_t stats[4] = {0, 0, 0, 0};
  if (which & 1)
    if (int rc = lines_direction(F, P, grad, 0, cells, stats, st)) return rc;
  if (which & 2)
    if (int rc = lines_direction(F, P, grad, 1, cells, stats, st)) return rc;
  if (stats_out)
    for (int k = 0; k < 4; k++) stats_out[k] = stats[k];
  return MSC_OK;
}

}  // namespace
}  // namespace msc

extern "C" int msc_saddle_lines_3d(const float* f, const uint8_t* grad, const uint32_t* zeroed, const int64_t dims[3],
                                   int which, const msc_integ_params* params, uint8_t* cells, int64_t stats[4],
                                   msc_stream_t stream) {
  return msc::saddle_lines_impl(f, grad, zeroed, dims, which, params, cells, stats, (cudaStream_t)stream);
}
