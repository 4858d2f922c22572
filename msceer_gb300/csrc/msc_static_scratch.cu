// The ascending-manifold (ldir) closure with its scratch in a static device array,
// for callers that may not allocate device memory.
//
// Some applications hand every byte of device memory out through their own pool or
// budget and forbid libraries from calling cudaMalloc behind their back (an
// allocation there would fail, or silently break the pool's accounting).  The
// regular msc_ascending_manifold_dims_3d asks the stream-ordered allocator for its
// per-pass tile flags; this variant keeps them in a fixed array that is part of the
// library image instead.
//
// The array (g_ldir_static) is a file-scope __device__ object: every GPU that loads
// the library holds it until the process exits.  Its host-side name is only a
// stand-in for the device object, so the host asks the runtime for the device
// address once per device (cudaGetSymbolAddress, with that device current) and
// passes that address to the kernels; the address is kept for the process, so the
// entry must not be used on a device after cudaDeviceReset there.  Every call shares
// the array and leaves the last call's contents in it; each call clears what must
// start at zero.  Two calls whose work overlaps on the GPU (e.g. on two streams) race
// on the shared array.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/msc_gpu.h"
#include "msc_device.cuh"

namespace msc {
int set_last_error(int code, const char* msg);
}

namespace {

// 1 MiB of tile flags: two halves (flags read / flags written by a pass), so at
// most 512 Ki tiles of 32x32x16 cells -- volumes up to about 1000^3 vertices.
constexpr int64_t kStaticFlagBytes = (int64_t)1 << 20;
constexpr int64_t kStaticMaxTiles = kStaticFlagBytes / 2;

struct LdirStaticScratch {
  int words[64];                     // [0] error bits, [1] "a pass changed a tile border"
  uint8_t flags[kStaticFlagBytes];
};

__device__ __align__(256) LdirStaticScratch g_ldir_static;

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
LdirStaticScratch* g_static_addr[kMaxDevices] = {};

// Device address of g_ldir_static on the current device (set up once per device).
int static_scratch(LdirStaticScratch** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return msc::set_last_error(MSC_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return msc::set_last_error(MSC_ERR_CUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_static_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_ldir_static);
    if (e != cudaSuccess || !p)
      return msc::set_last_error(MSC_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
    g_static_addr[dev] = static_cast<LdirStaticScratch*>(p);
  }
  *out = g_static_addr[dev];
  return MSC_OK;
}

}  // namespace

extern "C" int msc_ascending_manifold_dims_3d_static(uint8_t* grad, const int64_t dims[3], msc_stream_t stream,
                                                      int* passes_out) {
  if (!grad || !dims) return msc::set_last_error(MSC_ERR_NULL_POINTER, "null argument");
  msc::GradDims D{};
  if (!msc::make_grad_dims(3, dims, &D)) return msc::set_last_error(MSC_ERR_BAD_DIMS, "invalid dims");
  const int64_t ntiles = msc::ldir_num_tiles(3, D);
  if (ntiles <= 0) return msc::set_last_error(MSC_ERR_BAD_DIMS, "invalid dims");
  if (ntiles > kStaticMaxTiles) {
    const std::string m = "volume needs " + std::to_string(ntiles) + " ldir tiles; the static scratch holds " +
                          std::to_string(kStaticMaxTiles) + " (use msc_ascending_manifold_dims_3d)";
    return msc::set_last_error(MSC_ERR_TOO_LARGE, m.c_str());
  }
  LdirStaticScratch* S = nullptr;
  if (int rc = static_scratch(&S)) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 148;
  int* words = S->words;
  uint8_t* flags = S->flags;
  cudaError_t e = cudaMemsetAsync(words, 0, 2 * sizeof(int), st);
  if (e != cudaSuccess) return msc::set_last_error(MSC_ERR_CUDA, cudaGetErrorString(e));
  const int64_t limit = ntiles + 2;
  const uint8_t* din = nullptr;
  uint8_t* dout = flags;
  int passes = 0;
  while (true) {
    if ((e = cudaMemsetAsync(words + 1, 0, sizeof(int), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(dout, 0, (size_t)ntiles, st)) != cudaSuccess ||
        (e = msc::launch_ldir_pass(3, grad, D, din, dout, words + 1, words, sms, st)) != cudaSuccess)
      return msc::set_last_error(MSC_ERR_CUDA, cudaGetErrorString(e));
    passes++;
    int changed = 0;
    if ((e = cudaMemcpyAsync(&changed, words + 1, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return msc::set_last_error(MSC_ERR_CUDA, cudaGetErrorString(e));
    if (!changed) break;
    if (passes >= limit) return msc::set_last_error(MSC_ERR_ITER_LIMIT, "ldir closure did not converge");
    din = dout;
    dout = (dout == flags) ? flags + kStaticMaxTiles : flags;
  }
  int err = 0;
  if ((e = cudaMemcpyAsync(&err, words, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return msc::set_last_error(MSC_ERR_CUDA, cudaGetErrorString(e));
  if (err & msc::kErrLocalQueue) return msc::set_last_error(MSC_ERR_QUEUE_OVERFLOW, "ldir tile queue overflow");
  if (err & msc::kErrPassLimit) return msc::set_last_error(MSC_ERR_ITER_LIMIT, "ldir closure did not converge");
  if (passes_out) *passes_out = passes;
  return MSC_OK;
}
