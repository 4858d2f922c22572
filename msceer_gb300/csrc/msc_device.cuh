// Device-side definitions shared by the .grad kernels (sm_103a).
//
// The cell complex of an X x Y x Z vertex grid is the (2X-1)(2Y-1)(2Z-1) index
// lattice of TopologicalRegularGrid3D (gi_topological_regular_grid.h:113-126):
// cell (cx,cy,cz) has id cx + cy*dX + cz*dX*dY, dimension = number of odd
// coordinates, and vertex (x,y,z) is cell (2x,2y,2z).  One .grad byte per cell
// (GradBitfield, gi_discrete_gradient_labeling.h:11-19), LSB first:
//   bit 0 assigned, bit 1 flag (boundary), bits 2-4 pair direction
//   (0..5 = +x,-x,+y,-y,+z,-z, 7 = critical), bits 5-7 ldir.
#pragma once
#include <cstdint>

namespace msc {

// Process-wide count of the library's kernel launches (msc_kernel_launches()).
// The library's device scratch comes from a memory pool of its own per device that keeps
// its memory between calls (msc_trim_scratch hands the unused part back).
cudaError_t scratch_pool(cudaMemPool_t* out);
cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t stream);
// Records the calling thread's error text for msc_last_error_string(); returns code.
int set_last_error(int code, const char* msg);
void count_launch();
void add_launches(long long n);
long long launches_so_far();
// Labeling phase trace (MSC_LABELS_TRACE=1; msc_labels_capi.cu): a timing event on
// `st` at a phase boundary of direction `dir` (-1 ascending, 1 descending).
void label_trace(cudaStream_t st, int dir, const char* what);

enum : int {
  kErrNone = 0,
  kErrNaN = 1 << 0,          // input contains NaN (outside the order's contract)
  kErrPassLimit = 1 << 1,    // ldir closure did not converge within the pass bound
  kErrLocalQueue = 1 << 2,   // shared-memory BFS queue overflow (cannot happen by construction)
  kErrIterLimit = 1 << 3,    // a bounded walk hit its step limit (invalid gradient input)
};

struct GradDims {
  int64_t v[3];     // vertices per axis (v[2] = 1 in 2D)
  int64_t d[3];     // cells per axis, 2v-1
  int64_t cs[3];    // cell-id strides: 1, dX, dX*dY
  int64_t ncells;
  // local pair code (0..5 = +x,-x,+y,-y,+z,-z) -> code stored in the .grad byte.
  // Identity unless an axis has a single vertex, where the reference's encoder
  // (Compress6NeighborOffsetToByte, gi_topological_regular_grid.h:1182-1192)
  // reports the first axis whose stride is equal.  3 bits per code.
  uint32_t enc_map;
  // stored code -> true axis*2+sign, the inverse of enc_map for decoding.
  uint32_t dec_map;
};

__host__ __device__ inline int map3(uint32_t m, int c) { return (int)((m >> (3 * c)) & 7u); }

}  // namespace msc

#include <cuda_runtime.h>
namespace msc {
// launchers (defined next to their kernels)
cudaError_t launch_lstar(int nd, const float* f, uint8_t* g, const GradDims& D, int* err, int num_sms,
                         cudaStream_t stream);

// Batches of 3D volumes, passed by value in the launch parameters (no device table).
constexpr int kMaxBatch = 64;
struct LstarVol {
  const float* f;
  uint8_t* g;
  GradDims D;
  int64_t block0;  // first flat block of the volume
  int gx, gy;      // x-blocks per row, y-blocks per plane
};
struct LstarBatch {
  int n;
  int64_t total_blocks;
  LstarVol v[kMaxBatch];
};
cudaError_t make_lstar_batch(int n, const float* const* f, uint8_t* const* g, const GradDims* D, LstarBatch* B);
cudaError_t launch_lstar_batch(const LstarBatch& B, int* err, int num_sms, cudaStream_t stream,
                               int blocks_per_sm = 64);
// tiles of the multi-pass ldir kernel, and of the single-pass (bit-row) tile kernel
int64_t ldir_num_tiles(int nd, const GradDims& D);
int64_t ldir_bit_tiles(int nd, const GradDims& D);
// The mesh description of the C ABI's dims (false for invalid or overflowing dims),
// with the pair-code maps of single-vertex axes (msc_capi.cu).
bool make_grad_dims(int nd, const int64_t* dims, GradDims* D);
// halo record bytes of one single-pass tile
int64_t ldir_halo_bytes(int nd);
struct LdirVol {
  uint8_t* g;
  GradDims D;
  int64_t tile0;  // first flat tile of the volume
};
struct LdirBatch {
  int n;
  int64_t total_tiles;
  LdirVol v[kMaxBatch];
};
cudaError_t make_ldir_batch(int nd, int n, uint8_t* const* g, const GradDims* D, LdirBatch* B);
cudaError_t launch_ldir_tile(int nd, const LdirBatch& B, uint8_t* saved, int* err, int num_sms, cudaStream_t stream,
                             int ctas_per_sm = 4);
// one walk round whose input length is read from device memory (for graph capture)
cudaError_t launch_ldir_walk_dev(const LdirBatch& B, const int64_t* qin, const int* n_in_dev, int64_t* qout, int* n_out,
                                 int cap, int* lock, int* err, int num_sms, cudaStream_t stream);
cudaError_t launch_ldir_check(int nd, const LdirBatch& B, const uint8_t* saved, int64_t* queue, int* n_queue, int cap,
                              int* lock, int* err, int num_sms, cudaStream_t stream);
cudaError_t launch_ldir_walk(int nd, const LdirBatch& B, const int64_t* qin, int n_in, int64_t* qout, int* n_out,
                             int cap, int* lock, int* err, int num_sms, cudaStream_t stream);
cudaError_t launch_ldir_pass(int nd, uint8_t* g, const GradDims& D, const uint8_t* dirty_in, uint8_t* dirty_out,
                             int* changed, int* err, int num_sms, cudaStream_t stream);
cudaError_t launch_central_diff(int nd, int layout, const float* f, void* out, const GradDims& D, int num_sms,
                                cudaStream_t stream);
// Conforming gradient (conform_kernels.cu): restriction bytes per cell from the final
// ascending / descending labels (either may be null), then the re-pairing of the
// touched vertices (`touched` counts them) and every cell's ldir back to its roots.
cudaError_t launch_restriction_labels(const int32_t* asc, const int32_t* dsc, const float* f, const GradDims& D,
                                      uint8_t* out, int num_sms, cudaStream_t stream);
cudaError_t launch_conform(const float* f, const uint8_t* rlab, uint8_t* g, const GradDims& D,
                           unsigned long long* touched, int num_sms, cudaStream_t stream);
}  // namespace msc
