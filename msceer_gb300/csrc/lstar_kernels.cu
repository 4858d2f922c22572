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
// expands it on bitmasks.  Neighbour values live in a per-thread shared-memory
// column so the lowest-vertex comparisons can index them.  Each cell is owned by
// exactly one vertex (its highest), so its final byte is written once with a plain
// store; for one neighbour position the 32 stores of a warp fall in one 64-byte span.
#include "lstar_core.cuh"
#include "msc_device.cuh"

namespace msc {

__constant__ VertexMasks<3> c_vm3 = make_vertex_masks<3>();
__constant__ VertexMasks<2> c_vm2 = make_vertex_masks<2>();

// Block = BS threads = 32 consecutive x by BS/32 (y,z) rows; grid-stride over
// (x-block, row-block) pairs.
template <int ND, int BS>
__global__ void __launch_bounds__(BS) lstar_kernel(const float* __restrict__ f, uint8_t* __restrict__ g,
                                                   const GradDims D, int* __restrict__ err) {
  using N = Nb<ND>;
  constexpr int NPOS = N::NPOS;
  constexpr int ROWS = BS / 32;
  __shared__ float s_val[NPOS * BS];
  __shared__ uint32_t s_vm[NPOS];
  const int tid = threadIdx.x;
  if (tid < NPOS) s_vm[tid] = (ND == 3) ? c_vm3.vm[tid] : c_vm2.vm[tid];
  __syncthreads();

  const int64_t X = D.v[0], Y = D.v[1], Z = D.v[2];
  const int64_t nrows = Y * Z;
  const int64_t xblocks = (X + 31) / 32;
  const int64_t nblocks = xblocks * ((nrows + ROWS - 1) / ROWS);
  const int lane = tid & 31, row = tid >> 5;
  const int64_t cs1 = D.cs[1], cs2 = D.cs[2];
  float* col = s_val + tid;
  bool nan = false;

  for (int64_t blk = blockIdx.x; blk < nblocks; blk += gridDim.x) {
    const int64_t x = (blk % xblocks) * 32 + lane;
    const int64_t r = (blk / xblocks) * ROWS + row;
    if (x >= X || r >= nrows) continue;
    const int64_t y = r % Y, z = r / Y;
    const float* fv = f + (x + X * r);
    uint8_t* gc = g + (2 * x + 2 * y * cs1 + 2 * z * cs2);
    const int64_t XY = X * Y;
    auto load = [&](int p, float& v) {
      v = __ldg(fv + N::d(p, 0) + N::d(p, 1) * X + ((ND == 3) ? N::d(p, 2) : 0) * XY);
    };
    auto store = [&](int p, uint8_t b) {
      gc[N::d(p, 0) + N::d(p, 1) * cs1 + ((ND == 3) ? N::d(p, 2) : 0) * cs2] = b;
    };
    nan |= process_vertex<ND>(x, y, z, X, Y, Z, load, col, BS, s_vm, D.enc_map, store);
  }
  if (__any_sync(0xffffffffu, nan) && (tid & 31) == 0) atomicOr(err, kErrNaN);
}

cudaError_t launch_lstar(int nd, const float* f, uint8_t* g, const GradDims& D, int* err, int num_sms,
                         cudaStream_t stream) {
  constexpr int BS = 128;
  const int64_t rows = D.v[1] * D.v[2];
  const int64_t nblocks = ((D.v[0] + 31) / 32) * ((rows + BS / 32 - 1) / (BS / 32));
  const int64_t cap = (int64_t)num_sms * 16;
  const int grid = (int)(nblocks < cap ? nblocks : cap);
  if (grid <= 0) return cudaSuccess;
  if (nd == 3)
    lstar_kernel<3, BS><<<grid, BS, 0, stream>>>(f, g, D, err);
  else
    lstar_kernel<2, BS><<<grid, BS, 0, stream>>>(f, g, D, err);
  return cudaGetLastError();
}

}  // namespace msc
