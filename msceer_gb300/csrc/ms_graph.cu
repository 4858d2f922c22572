// The Morse-Smale complex graph of a device-resident .grad: the nodes and arcs
// MorseSmaleComplexBasic::ComputeFromGrad builds without arc geometry
// (gi_morse_smale_complex_basic.h:676-716), as extractmsc uses it after load_from_file
// (extractmsc/extractmsc.cxx:482-504), read from the .grad in HBM instead of a file.
//
//   nodes  every critical cell (pair code 7) in cell-id order (AllCellsIterator):
//          cell id, dimension, boundaryValue, value = f at the cell's highest vertex
//          (createNode, :308-341, with TopologicalMaxVertexMeshFunction::cellValue)
//   arcs   for every node of dimension d >= 1 whose arcs are built (build[d - 1]),
//          the V-paths traced down from it (rec_tdcr_candidates, :550-577): a critical
//          facet ends a path in an arc to that facet's node; a facet whose ldir equals
//          the node's ldir + 1 continues at its pair when the pair is another cell of
//          the traced cell's dimension.  Arcs are listed node by node (the reference's
//          thread-local candidate lists, concatenated in thread order over a static
//          split of the nodes) and, within a node, in depth-first facet order
//          (+x, -x, +y, -y, +z, -z over the cell's odd axes); a path reached twice is
//          an arc twice.  persistence = value(upper) - value(lower) (createArcFromNodeIDs).
//
// GPU form: an ordered compaction of the critical cells (block counts, one scan, an
// ordered write), one thread per node for the attributes, and two depth-first passes
// per node thread -- one counts its arcs, a scan places them, one writes them -- with
// an explicit task stack: a visited cell pushes its children (arc ends and cells to
// visit) in reverse facet order, so a path without branches keeps the stack flat.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/msc_gpu.h"
#include "msc_device.cuh"

namespace msc {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kCritThreads = 256;
constexpr int kCritPerThread = 16;
constexpr int64_t kCritChunk = (int64_t)kCritThreads * kCritPerThread;  // cells per block
constexpr int kStack = 64;            // pending tasks of one node's trace
// cells one node's trace may visit: a valid .grad is acyclic, so this only stops the
// endless walk of a .grad with a cycle (a corrupt file, or one read with wrong dims)
constexpr int64_t kMaxVisits = (int64_t)1 << 24;
constexpr int64_t kEmit = (int64_t)1 << 62;  // task tag: an arc to the critical cell

struct MsMesh {
  const uint8_t* g;
  const float* f;
  int64_t d[3], cs[3], v[3];
  int64_t ncells;
  bool i32;  // cell ids fit 32 bits
};

__device__ __forceinline__ bool crit(uint8_t b) { return ((b >> 2) & 7u) == 7u; }
__device__ __forceinline__ int ldir(uint8_t b) { return b >> 5; }

__device__ __forceinline__ void coords(const MsMesh& M, int64_t id, int64_t c[3]) {
  if (M.i32) {
    const uint32_t u = (uint32_t)id, d0 = (uint32_t)M.d[0], d1 = (uint32_t)M.d[1];
    const uint32_t r = u / d0;
    c[0] = u - r * d0;
    c[1] = r % d1;
    c[2] = r / d1;
  } else {
    c[0] = id % M.d[0];
    c[1] = (id / M.d[0]) % M.d[1];
    c[2] = id / (M.d[0] * M.d[1]);
  }
}
__device__ __forceinline__ int dim_of(const int64_t c[3]) { return (int)((c[0] & 1) + (c[1] & 1) + (c[2] & 1)); }

// block-wide exclusive scan of one value per thread (blockDim.x threads, a multiple
// of 32); returns the thread's offset, *total the block's sum
template <class T>
__device__ T block_excl_scan(T v, T* s_warp, T* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? s_warp[lane] : (T)0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) s_warp[lane] = w;
  }
  __syncthreads();
  const T before = (warp > 0 ? s_warp[warp - 1] : (T)0) + x - v;
  if (total) *total = s_warp[nw - 1];
  __syncthreads();
  return before;
}

// the critical-cell bits of a thread's 16 cells (one 16-byte load when aligned)
__device__ __forceinline__ uint32_t crit_bits(const uint8_t* g, int64_t ncells, int64_t base) {
  uint32_t m = 0;
  if (base + 16 <= ncells && ((reinterpret_cast<uintptr_t>(g + base) & 15u) == 0)) {
    const uint4 q = *reinterpret_cast<const uint4*>(g + base);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 16; k++) m |= (uint32_t)crit((uint8_t)(w[k >> 2] >> (8 * (k & 3)))) << k;
  } else {
    for (int k = 0; k < 16; k++)
      if (base + k < ncells) m |= (uint32_t)crit(g[base + k]) << k;
  }
  return m;
}

__global__ void __launch_bounds__(kCritThreads) crit_count_kernel(const uint8_t* __restrict__ g, int64_t ncells,
                                                                  int64_t* __restrict__ counts) {
  __shared__ int64_t s_warp[32];
  const int64_t base = (int64_t)blockIdx.x * kCritChunk + (int64_t)threadIdx.x * kCritPerThread;
  int64_t total = 0;
  block_excl_scan<int64_t>(__popc(crit_bits(g, ncells, base)), s_warp, &total);
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

// in place: counts[0, n) -> exclusive offsets; *sum = the total.  One block.
template <class T>
__global__ void __launch_bounds__(kScanThreads) excl_scan_kernel(T* __restrict__ a, int64_t n, T* __restrict__ sum) {
  __shared__ T s_warp[32];
  T carry = 0;
  for (int64_t i0 = 0; i0 < n; i0 += kScanThreads) {
    const int64_t i = i0 + threadIdx.x;
    const T v = i < n ? a[i] : (T)0;
    T tot = 0;
    const T off = block_excl_scan<T>(v, s_warp, &tot);
    if (i < n) a[i] = carry + off;
    carry += tot;
  }
  if (threadIdx.x == 0) *sum = carry;
}

// The same for long arrays, in three launches: the sum of every kScanThreads-element
// chunk, the one-block scan of those sums, then every chunk scanned from its offset.
template <class T>
__global__ void __launch_bounds__(kScanThreads) chunk_sum_kernel(const T* __restrict__ a, int64_t n,
                                                                 T* __restrict__ sums) {
  __shared__ T s_warp[32];
  const int64_t i = (int64_t)blockIdx.x * kScanThreads + threadIdx.x;
  T tot = 0;
  block_excl_scan<T>(i < n ? a[i] : (T)0, s_warp, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}
template <class T>
__global__ void __launch_bounds__(kScanThreads) chunk_scan_kernel(T* __restrict__ a, int64_t n,
                                                                  const T* __restrict__ offs) {
  __shared__ T s_warp[32];
  const int64_t i = (int64_t)blockIdx.x * kScanThreads + threadIdx.x;
  const T v = i < n ? a[i] : (T)0;
  const T off = block_excl_scan<T>(v, s_warp, nullptr);
  if (i < n) a[i] = offs[blockIdx.x] + off;
}

__global__ void __launch_bounds__(kCritThreads) crit_write_kernel(const uint8_t* __restrict__ g, int64_t ncells,
                                                                  const int64_t* __restrict__ offsets,
                                                                  int64_t* __restrict__ node_cell) {
  __shared__ int64_t s_warp[32];
  const int64_t base = (int64_t)blockIdx.x * kCritChunk + (int64_t)threadIdx.x * kCritPerThread;
  uint32_t m = crit_bits(g, ncells, base);
  int64_t o = offsets[blockIdx.x] + block_excl_scan<int64_t>(__popc(m), s_warp, nullptr);
  while (m) {
    const int k = __ffs(m) - 1;
    m &= m - 1;
    node_cell[o++] = base + k;
  }
}

// createNode: dimension, boundaryValue and the value at the highest vertex ((value,
// then index) order, gi_regular_grid_trilinear_function.h:309-314)
__global__ void node_attr_kernel(const MsMesh M, const int64_t* __restrict__ node_cell, int64_t n,
                                 float* __restrict__ value, uint8_t* __restrict__ dim, uint8_t* __restrict__ bnd) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t c[3];
    coords(M, node_cell[i], c);
    int nb = 0;
    for (int a = 0; a < 3; a++) nb += (c[a] == 0 || c[a] == M.d[a] - 1);
    int64_t best = -1;
    float bv = 0.f;
    const int odd = (int)(c[0] & 1) | (int)((c[1] & 1) << 1) | (int)((c[2] & 1) << 2);
    for (int s = 0; s < 8; s++) {
      if (s & ~odd) continue;  // corners only along the odd axes
      int64_t vi = 0;
      for (int a = 0; a < 3; a++) {
        const int64_t vc = (c[a] & 1) ? ((s >> a) & 1 ? (c[a] + 1) >> 1 : (c[a] - 1) >> 1) : c[a] >> 1;
        vi += vc * M.v[a];
      }
      const float fv = M.f[vi];
      if (best < 0 || fv > bv || (!(bv > fv) && vi > best)) {
        best = vi;
        bv = fv;
      }
    }
    value[i] = bv;
    dim[i] = (uint8_t)dim_of(c);
    bnd[i] = (uint8_t)nb;
  }
}

__device__ __forceinline__ int64_t node_of(const int64_t* __restrict__ node_cell, int64_t n, int64_t cell) {
  int64_t lo = 0, hi = n - 1;
  while (lo <= hi) {
    const int64_t mid = (lo + hi) >> 1;
    const int64_t v = node_cell[mid];
    if (v == cell) return mid;
    if (v < cell) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

// One node's trace (rec_tdcr_candidates): counts its arcs, or writes them from `out`.
// Returns 0, kErrLocalQueue if the task stack overflowed, kErrIterLimit past kMaxVisits.
template <bool WRITE>
__device__ int trace_node(const MsMesh& M, const int64_t* __restrict__ node_cell, int64_t n, int64_t node,
                           int64_t* count, int64_t out, const float* __restrict__ value, int32_t* __restrict__ lower,
                           int32_t* __restrict__ upper, float* __restrict__ pers) {
  const int64_t start = node_cell[node];
  const int temp_dim = ldir(M.g[start]) + 1;
  int64_t stack[kStack];
  int sp = 0;
  stack[sp++] = start;
  int64_t k = 0, visits = 0;
  while (sp > 0) {
    const int64_t t = stack[--sp];
    if (t & kEmit) {
      if (WRITE) {
        const int64_t lo = node_of(node_cell, n, t & ~kEmit);
        lower[out + k] = (int32_t)lo;
        upper[out + k] = (int32_t)node;
        if (pers) pers[out + k] = value[node] - value[lo];
      }
      k++;
      continue;
    }
    if (++visits > kMaxVisits) return kErrIterLimit;
    int64_t c[3];
    coords(M, t, c);
    const int dim = dim_of(c);
    int64_t child[6];
    int nc = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      if (!(c[a] & 1)) continue;
#pragma unroll
      for (int s = 0; s < 2; s++) {
        const int64_t fc = s == 0 ? t + M.cs[a] : t - M.cs[a];
        const uint8_t b = M.g[fc];
        const unsigned code = (b >> 2) & 7u;
        if (code == 7u) {
          child[nc++] = fc | kEmit;
        } else if (code < 6u && ldir(b) == temp_dim) {
          // the pair: the cell at the code's stride (UncompressByteTo6NeighborOffset;
          // with a single-vertex axis two axes share a stride and the code names the
          // first), inside the array for any byte
          const int64_t p = (code & 1u) ? fc - M.cs[code >> 1] : fc + M.cs[code >> 1];
          if (p == t || p < 0 || p >= M.ncells) continue;
          int64_t pc[3];
          coords(M, p, pc);
          if (dim_of(pc) == dim) child[nc++] = p;
        }
      }
    }
    if (sp + nc > kStack) return kErrLocalQueue;
    for (int i = nc - 1; i >= 0; i--) stack[sp++] = child[i];
  }
  *count = k;
  return 0;
}

// The nodes whose arcs are traced (dimension d >= 1 with build bit d - 1), listed so
// that the tracing threads of a warp all trace (in cell order a warp's nodes mix all
// four dimensions, and minima and unbuilt dimensions left most lanes idle).
__global__ void traced_list_kernel(const MsMesh M, const int64_t* __restrict__ node_cell, int64_t n, int build,
                                   int32_t* __restrict__ list, unsigned long long* __restrict__ n_list) {
  const int lane = threadIdx.x & 31;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x; i0 < n; i0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = i0 + threadIdx.x;
    bool want = false;
    if (i < n) {
      int64_t c[3];
      coords(M, node_cell[i], c);
      const int d = dim_of(c);
      want = d > 0 && ((build >> (d - 1)) & 1);
    }
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) continue;
    const int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(n_list, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (want) list[base + __popc(m & ((1u << lane) - 1u))] = (int32_t)i;
  }
}

__global__ void arc_count_kernel(const MsMesh M, const int64_t* __restrict__ node_cell, int64_t n,
                                 const int32_t* __restrict__ list, const unsigned long long* __restrict__ n_list,
                                 int64_t* __restrict__ counts, int* __restrict__ err) {
  const int64_t nl = (int64_t)*n_list;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nl; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = list[j];
    int64_t k = 0;
    const int e = trace_node<false>(M, node_cell, n, i, &k, 0, nullptr, nullptr, nullptr, nullptr);
    if (e) {
      atomicOr(err, e);
      k = 0;
    }
    counts[i] = k;
  }
}

__global__ void arc_write_kernel(const MsMesh M, const int64_t* __restrict__ node_cell, int64_t n,
                                 const int32_t* __restrict__ list, const unsigned long long* __restrict__ n_list,
                                 const int64_t* __restrict__ offsets, const float* __restrict__ value,
                                 int32_t* __restrict__ lower, int32_t* __restrict__ upper, float* __restrict__ pers,
                                 int* __restrict__ err) {
  const int64_t nl = (int64_t)*n_list;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nl; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = list[j];
    int64_t k = 0;
    const int e = trace_node<true>(M, node_cell, n, i, &k, offsets[i], value, lower, upper, pers);
    if (e) atomicOr(err, e);
  }
}

int fail(int code, const std::string& m) { return set_last_error(code, m.c_str()); }
#define GCUDA(call, what)                                                                          \
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
  cudaError_t get(void** out, size_t bytes) {
    cudaError_t e = scratch_alloc(out, bytes ? bytes : 16, st);
    if (e == cudaSuccess) p.push_back(*out);
    return e;
  }
};

int grid_for(int64_t n, int threads) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)sms * 16;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

// a[0, n) -> exclusive offsets in place, *sum (device) = the total
int scan_in_place(Pool& P, int64_t* a, int64_t n, int64_t* sum, cudaStream_t stream) {
  const int64_t nch = (n + kScanThreads - 1) / kScanThreads;
  int64_t* csum = nullptr;
  GCUDA(P.get((void**)&csum, (size_t)(nch + 1) * sizeof(int64_t)), "scratch alloc(chunk sums)");
  if (nch > 0) {
    count_launch();
    chunk_sum_kernel<int64_t><<<(unsigned)nch, kScanThreads, 0, stream>>>(a, n, csum);
  }
  count_launch();
  excl_scan_kernel<int64_t><<<1, kScanThreads, 0, stream>>>(csum, nch, sum);
  if (nch > 0) {
    count_launch();
    chunk_scan_kernel<int64_t><<<(unsigned)nch, kScanThreads, 0, stream>>>(a, n, csum);
  }
  return MSC_OK;
}

int ms_graph_impl(const uint8_t* g, const float* f, const int64_t* dims, const int* build, int64_t node_cap,
                  int64_t* node_cell, float* node_value, uint8_t* node_dim, uint8_t* node_boundary, int64_t arc_cap,
                  int32_t* arc_lower, int32_t* arc_upper, float* arc_pers, int64_t* counts_out,
                  cudaStream_t stream) {
  if (!dims || !build || !counts_out) return fail(MSC_ERR_NULL_POINTER, "null argument");
  GradDims D;
  if (!make_grad_dims(3, dims, &D)) return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  if (!g || !f) return fail(MSC_ERR_NULL_POINTER, "null buffer");
  MsMesh M;
  M.g = g;
  M.f = f;
  for (int a = 0; a < 3; a++) {
    M.d[a] = D.d[a];
    M.cs[a] = D.cs[a];
  }
  M.v[0] = 1;
  M.v[1] = D.v[0];
  M.v[2] = D.v[0] * D.v[1];
  M.ncells = D.ncells;
  M.i32 = D.ncells <= (int64_t)0xFFFFFFFF;
  const int bmask = (build[0] ? 1 : 0) | (build[1] ? 2 : 0) | (build[2] ? 4 : 0);

  Pool P{{}, stream};
  const int64_t nblk = (D.ncells + kCritChunk - 1) / kCritChunk;
  int64_t* blk = nullptr;
  int64_t* sums = nullptr;  // [0] nodes [1] arcs
  int* err = nullptr;
  GCUDA(P.get((void**)&blk, (size_t)nblk * sizeof(int64_t)), "scratch alloc(block counts)");
  GCUDA(P.get((void**)&sums, 2 * sizeof(int64_t) + sizeof(int)), "scratch alloc(sums)");
  err = reinterpret_cast<int*>(sums + 2);
  GCUDA(cudaMemsetAsync(err, 0, sizeof(int), stream), "cudaMemsetAsync(status)");
  count_launch();
  crit_count_kernel<<<(unsigned)nblk, kCritThreads, 0, stream>>>(g, D.ncells, blk);
  if (int rc = scan_in_place(P, blk, nblk, sums, stream)) return rc;
  GCUDA(cudaGetLastError(), "critical-cell count launch");
  int64_t h[2] = {0, 0};
  GCUDA(cudaMemcpyAsync(h, sums, sizeof(int64_t), cudaMemcpyDeviceToHost, stream), "read node count");
  GCUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  const int64_t n = h[0];
  if (n >= ((int64_t)1 << 31)) return fail(MSC_ERR_BAD_DIMS, "more than 2^31 - 1 critical cells");

  const bool nodes_out = node_cell && node_value && node_dim && node_boundary && node_cap >= n;
  int64_t* cells = node_cell;
  float* vals = node_value;
  if (!nodes_out) {
    GCUDA(P.get((void**)&cells, (size_t)n * sizeof(int64_t)), "scratch alloc(node cells)");
    GCUDA(P.get((void**)&vals, (size_t)n * sizeof(float)), "scratch alloc(node values)");
  }
  count_launch();
  crit_write_kernel<<<(unsigned)nblk, kCritThreads, 0, stream>>>(g, D.ncells, blk, cells);
  int64_t* acnt = nullptr;
  int32_t* tlist = nullptr;
  unsigned long long* n_tlist = nullptr;
  GCUDA(P.get((void**)&acnt, (size_t)n * sizeof(int64_t)), "scratch alloc(arc counts)");
  GCUDA(P.get((void**)&tlist, (size_t)n * sizeof(int32_t)), "scratch alloc(traced nodes)");
  GCUDA(P.get((void**)&n_tlist, sizeof(unsigned long long)), "scratch alloc(traced count)");
  GCUDA(cudaMemsetAsync(acnt, 0, (size_t)n * sizeof(int64_t), stream), "cudaMemsetAsync(arc counts)");
  GCUDA(cudaMemsetAsync(n_tlist, 0, sizeof(unsigned long long), stream), "cudaMemsetAsync(traced count)");
  if (n > 0) {
    count_launch();
    traced_list_kernel<<<grid_for(n, 256), 256, 0, stream>>>(M, cells, n, bmask, tlist, n_tlist);
    count_launch();
    arc_count_kernel<<<grid_for(n, 128), 128, 0, stream>>>(M, cells, n, tlist, n_tlist, acnt, err);
  }
  if (int rc = scan_in_place(P, acnt, n, sums + 1, stream)) return rc;
  GCUDA(cudaGetLastError(), "arc count launch");
  int st = 0;
  GCUDA(cudaMemcpyAsync(h + 1, sums + 1, sizeof(int64_t), cudaMemcpyDeviceToHost, stream), "read arc count");
  GCUDA(cudaMemcpyAsync(&st, err, sizeof(int), cudaMemcpyDeviceToHost, stream), "read status");
  GCUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  if (st & kErrIterLimit) return fail(MSC_ERR_ITER_LIMIT, "a V-path trace did not end (is the .grad acyclic?)");
  if (st) return fail(MSC_ERR_QUEUE_OVERFLOW, "a V-path trace branched beyond its task stack");
  const int64_t na = h[1];
  counts_out[0] = n;
  counts_out[1] = na;

  const bool arcs_out = arc_lower && arc_upper && arc_cap >= na;
  if (!nodes_out && !arcs_out) return MSC_OK;
  uint8_t* dims_b = node_dim;
  uint8_t* bnd_b = node_boundary;
  if (!nodes_out) {
    GCUDA(P.get((void**)&dims_b, (size_t)n), "scratch alloc(node dims)");
    GCUDA(P.get((void**)&bnd_b, (size_t)n), "scratch alloc(node boundary)");
  }
  if (n > 0) {
    count_launch();
    node_attr_kernel<<<grid_for(n, 256), 256, 0, stream>>>(M, cells, n, vals, dims_b, bnd_b);
  }
  if (arcs_out && n > 0) {
    count_launch();
    arc_write_kernel<<<grid_for(n, 128), 128, 0, stream>>>(M, cells, n, tlist, n_tlist, acnt, vals, arc_lower,
                                                           arc_upper, arc_pers, err);
  }
  GCUDA(cudaGetLastError(), "node / arc write launch");
  GCUDA(cudaMemcpyAsync(&st, err, sizeof(int), cudaMemcpyDeviceToHost, stream), "read status");
  GCUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  if (st & kErrIterLimit) return fail(MSC_ERR_ITER_LIMIT, "a V-path trace did not end (is the .grad acyclic?)");
  if (st) return fail(MSC_ERR_QUEUE_OVERFLOW, "a V-path trace branched beyond its task stack");
  return MSC_OK;
}

}  // namespace
}  // namespace msc

extern "C" {

int msc_ms_graph_3d(const uint8_t* grad, const float* f, const int64_t dims[3], const int build_arcs[3],
                    int64_t node_cap, int64_t* node_cell, float* node_value, uint8_t* node_dim,
                    uint8_t* node_boundary, int64_t arc_cap, int32_t* arc_lower, int32_t* arc_upper,
                    float* arc_persistence, int64_t counts[2], msc_stream_t stream) {
  return msc::ms_graph_impl(grad, f, dims, build_arcs, node_cap, node_cell, node_value, node_dim, node_boundary,
                            arc_cap, arc_lower, arc_upper, arc_persistence, counts,
                            reinterpret_cast<cudaStream_t>(stream));
}

}  // extern "C"
