// K1: lower-star discrete gradient, one thread per vertex (sm_103a).
//
// Replaces, with identical output bytes:
//   RegularGridMaxMinVertexLabeling3D::ComputeOutput   gi_max_vertex_labeling.h:1119-1339
//   SlidingWindowRobinsNoalloc::ComputePairing_sliding gi_fast_robins_noalloc.h:1254-1535
//     (interior: ComputeLowerStar :353-428, HomotopyExpand :147-321)
//   MyRobinsNoalloc<...,5,4>::ComputeLowerStar          gi_modified_robins.h:1281-1343
//     (boundary planes, lower star split by cell boundaryValue)
//   2D: RegularGridMaxMinVertexLabeling2D + MyRobinsNoalloc<TopologicalRegularGrid2D,...,4,6>
//       ::ComputePairing (gi_modified_robins.h:1344-1402)
// and the parts of setAscendingManifoldDimensions / outputToFile that are local to a
// cell: the boundary flag and the ldir value of critical cells (the roots of the
// ascending-manifold closure, finished by ldir_kernels.cu).
//
// The max/min vertex labeling is never materialised: the per-vertex work
// (lstar_core.cuh) derives the lower star from the neighbours below the vertex and
// expands it on bitmasks.  The lowest-vertex key of every cell of the neighbourhood
// lives in a per-thread shared-memory column so the comparisons can index it.  Each
// cell is owned by exactly one vertex (its highest), so its final byte is written
// once with a plain store; for one neighbour position the 32 stores of a warp fall in
// one 64-byte span.
#include "lstar_core.cuh"
#include "msc_device.cuh"

namespace msc {

// One block's work: 32 consecutive x by BS/32 consecutive y at one z of volume (f, g,
// D).  Neighbour and cell offsets are 32-bit; only the per-vertex base addresses are
// 64-bit.  Every thread first builds its own vertex's keys and lower star; the
// expansions -- whose loop runs once per pairing step, so its length follows the
// lower star's size -- are then handed out in order of that size, so that the lanes
// of a warp run loops of similar length (one thread per vertex otherwise left half the
// lanes idle).  Every thread of the block must call this (it synchronises the block).
template <int ND, int BS>
__device__ __forceinline__ bool lstar_block(const float* __restrict__ f, uint8_t* __restrict__ g, const GradDims& D,
                                            int64_t bx, int64_t by, int64_t z, uint64_t* s_key, uint32_t* s_L,
                                            int* s_order, int* s_hist) {
  using N = Nb<ND>;
  constexpr int ROWS = BS / 32;
  const int tid = threadIdx.x;
  const int64_t X = D.v[0], Y = D.v[1], Z = D.v[2];
  const int sX = (int)X, sXY = (int)(X * Y);
  const int c1 = (int)D.cs[1], c2 = (int)D.cs[2];
  auto vertex = [&](int t, int64_t& x, int64_t& y) {
    x = bx * 32 + (t & 31);
    y = by * ROWS + (t >> 5);
    return x < X && y < Y;
  };
  auto is_interior = [&](int64_t x, int64_t y) {
    return x > 0 && x < X - 1 && y > 0 && y < Y - 1 && (ND == 2 || (z > 0 && z < Z - 1));
  };
  if (tid < 32) s_hist[tid] = 0;
  __syncthreads();
  int64_t x, y;
  bool nan = false;
  int size = -1;  // popcount of the lower star; -1: no vertex here
  if (vertex(tid, x, y)) {
    const float* fv = f + (x + X * (y + Y * z));
    auto load = [&](int p, float& v) {
      v = __ldg(fv + (N::d(p, 0) + N::d(p, 1) * sX + (ND == 3 ? N::d(p, 2) : 0) * sXY));
    };
    const uint32_t L = lower_star_keys<ND>(x, y, z, X, Y, Z, is_interior(x, y), load, s_key + tid, BS, nan);
    s_L[tid] = L;
    size = __popc(L);
  }
  // counting sort of the block's vertices by lower-star size (28 sizes)
  const int bin = size < 0 ? 31 : size;
  const int rank = atomicAdd(&s_hist[bin], 1);
  __syncthreads();
  if (tid < 32) {
    const int c = s_hist[tid];
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (tid >= o) incl += u;
    }
    s_hist[tid] = incl - c;  // exclusive start of each bin
  }
  __syncthreads();
  s_order[s_hist[bin] + rank] = tid;
  __syncthreads();
  const int t = s_order[tid];
  if (vertex(t, x, y)) {
    uint8_t* gc = g + (2 * x + 2 * y * D.cs[1] + 2 * z * D.cs[2]);
    auto store = [&](int p, uint8_t b) { gc[N::d(p, 0) + N::d(p, 1) * c1 + (ND == 3 ? N::d(p, 2) : 0) * c2] = b; };
    expand_and_store<ND>(s_L[t], s_key + t, BS, is_interior(x, y), x == 0 || x == X - 1, y == 0 || y == Y - 1,
                         z == 0 || z == Z - 1, D.enc_map, store);
  }
  __syncthreads();  // the keys and masks are reused for the next z
  return nan;
}

// One volume: grid (x-blocks, y-blocks, z), looping over z when Z exceeds the grid.
template <int ND, int BS>
__global__ void __launch_bounds__(BS) lstar_kernel(const float* __restrict__ f, uint8_t* __restrict__ g,
                                                   const GradDims D, int* __restrict__ err) {
  __shared__ uint64_t s_key[Nb<ND>::NPOS * BS];
  __shared__ uint32_t s_L[BS];
  __shared__ int s_order[BS], s_hist[32];
  bool nan = false;
  for (int64_t z = blockIdx.z; z < D.v[2]; z += gridDim.z)
    nan |= lstar_block<ND, BS>(f, g, D, blockIdx.x, blockIdx.y, z, s_key, s_L, s_order, s_hist);
  if (nan) atomicOr(err, kErrNaN);
}

// Many volumes in one launch: a flat grid over every volume's (x-block, y-block, z)
// triples; a block finds its volume by binary search over the volumes' first blocks.
template <int BS>
__global__ void __launch_bounds__(BS) lstar_batch_kernel(const LstarBatch B, int* __restrict__ err) {
  __shared__ uint64_t s_key[27 * BS];
  __shared__ uint32_t s_L[BS];
  __shared__ int s_order[BS], s_hist[32];
  bool nan = false;
  for (int64_t blk = blockIdx.x; blk < B.total_blocks; blk += gridDim.x) {
    int lo = 0, hi = B.n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (B.v[mid].block0 <= blk) lo = mid; else hi = mid - 1;
    }
    const LstarVol& V = B.v[lo];
    const int64_t r = blk - V.block0;
    const int64_t bx = r % V.gx, by = (r / V.gx) % V.gy, z = r / ((int64_t)V.gx * V.gy);
    nan |= lstar_block<3, BS>(V.f, V.g, V.D, bx, by, z, s_key, s_L, s_order, s_hist);
  }
  if (nan) atomicOr(err, kErrNaN);
}

namespace {
constexpr int kLstarBS = 128;
bool lstar_dims_ok(const GradDims& D) {
  // a z-plane of cells must be addressable with 32-bit offsets
  return !(D.v[0] > (int64_t)1 << 30 || D.v[1] > (int64_t)1 << 30 || D.v[0] * D.v[1] > ((int64_t)1 << 31) - 1 ||
           D.cs[2] > ((int64_t)1 << 31) - 1);
}
}  // namespace

cudaError_t launch_lstar(int nd, const float* f, uint8_t* g, const GradDims& D, int* err, int num_sms,
                         cudaStream_t stream) {
  (void)num_sms;
  constexpr int BS = kLstarBS;
  if (!lstar_dims_ok(D)) return cudaErrorInvalidValue;
  const dim3 grid((unsigned)((D.v[0] + 31) / 32), (unsigned)((D.v[1] + BS / 32 - 1) / (BS / 32)),
                  (unsigned)(D.v[2] < 65535 ? D.v[2] : 65535));
  if (grid.y > 65535u) return cudaErrorInvalidValue;
  if (nd == 3) {
    ::msc::count_launch();
    lstar_kernel<3, BS><<<grid, BS, 0, stream>>>(f, g, D, err);
  } else {
    ::msc::count_launch();
    lstar_kernel<2, BS><<<grid, BS, 0, stream>>>(f, g, D, err);
  }
  return cudaGetLastError();
}

cudaError_t make_lstar_batch(int n, const float* const* f, uint8_t* const* g, const GradDims* D, LstarBatch* B) {
  if (n < 1 || n > kMaxBatch) return cudaErrorInvalidValue;
  B->n = n;
  int64_t off = 0;
  for (int i = 0; i < n; i++) {
    if (!lstar_dims_ok(D[i])) return cudaErrorInvalidValue;
    LstarVol& v = B->v[i];
    v.f = f[i];
    v.g = g[i];
    v.D = D[i];
    v.gx = (int)((D[i].v[0] + 31) / 32);
    v.gy = (int)((D[i].v[1] + kLstarBS / 32 - 1) / (kLstarBS / 32));
    v.block0 = off;
    off += (int64_t)v.gx * v.gy * D[i].v[2];
  }
  B->total_blocks = off;
  return cudaSuccess;
}

cudaError_t launch_lstar_batch(const LstarBatch& B, int* err, int num_sms, cudaStream_t stream, int blocks_per_sm) {
  const int64_t cap = (int64_t)num_sms * blocks_per_sm;
  const int grid = (int)(B.total_blocks < cap ? B.total_blocks : cap);
  if (grid <= 0) return cudaSuccess;
  ::msc::count_launch();
  lstar_batch_kernel<kLstarBS><<<grid, kLstarBS, 0, stream>>>(B, err);
  return cudaGetLastError();
}

}  // namespace msc
