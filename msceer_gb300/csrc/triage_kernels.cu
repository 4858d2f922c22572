// Learned triage: a 3x3x3 convolutional network (Cin -> 16 -> 16 -> 2 channels) that
// flags the vertices whose integrated destination differs from their combinatorial
// steepest-path destination.  Forward and input-gradient convolutions are BF16
// implicit GEMMs on the tcgen05 tensor cores with FP32 accumulation in TMEM; the
// weight gradient, loss and optimiser run on the CUDA cores in FP32.
//
// Activation layout ("row-planar"): [Z][Y][2][X][8] BF16.  Each (y, z) row of the
// volume holds two planes, channels 0-7 and channels 8-15, each X x 16 bytes.  That
// is the K-major, no-swizzle operand layout of the MMA (8-row x 16-byte core
// matrices, rows 16 bytes apart), so an A operand is a plain address into a staged
// row: output vertices x0..x0+127 under tap (dx, dy, dz) read the staged row of
// (y+dy, z+dz) starting at x0+dx.
//
// One CTA computes a 128 (x) x 4 (y) block of output rows at one z: a single TMA
// load stages the 130 x 6 x 3 input rows (zero fill outside the volume = zero
// padding), a bulk copy stages the 27 weight taps, one thread issues the 4 x 27
// MMAs (M=128 vertices, N=16 output channels, K=16 input channels each) into four
// TMEM accumulators, and four warps read them back for the epilogue.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "tc_sm100.cuh"
#include "triage.cuh"

namespace msc {

namespace {
constexpr int kBX = 128;  // output vertices per row (MMA M)
constexpr int kBY = 4;    // output rows per CTA (along y)
constexpr int kInY = kBY + 2, kInZ = 3;
constexpr int kPlaneB = (kBX + 2) * 16;             // one staged 8-channel plane
constexpr int kRowB = 2 * kPlaneB;                  // one staged row
constexpr int kStageB = kRowB * kInY * kInZ;        // the TMA box
constexpr int kTapB = 512;                          // 16 x 16 BF16 weights of one tap
constexpr int kWeightB = 27 * kTapB;
constexpr int kSmemConv = 1024 + kStageB + kWeightB + 64;
constexpr uint32_t kTmemCols = 64;                  // 4 accumulators of 16 columns
static_assert(kStageB % 16 == 0 && kWeightB % 16 == 0, "bulk copy sizes");
static_assert(kBY * 16 <= (int)kTmemCols, "accumulators fit the allocation");
}  // namespace

__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
      "[%7];" ::"r"(tc::smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(tc::smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tc::smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Epilogue kinds
//   kEpiReluBf16  out = bf16(relu(acc + bias))                         (hidden layers)
//   kEpiLogits    logits[c][v] = acc[c] + bias[c], c < 2, FP32 planar  (output layer)
//   kEpiMaskBf16  out = bf16(acc * (mask_act > 0))                     (input gradient)
template <int EPI>
__global__ void __launch_bounds__(128) conv3_tc_kernel(const __grid_constant__ CUtensorMap in_map,
                                                       const uint8_t* __restrict__ wblob, const float* __restrict__ bias,
                                                       const ConvDims D, __nv_bfloat16* __restrict__ out_act,
                                                       float* __restrict__ out_logits,
                                                       const __nv_bfloat16* __restrict__ mask_act, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* s_in = sm;
  unsigned char* s_w = sm + kStageB;
  uint64_t* bars = reinterpret_cast<uint64_t*>(s_w + kWeightB);  // [0] loads, [1] mma
  uint32_t* s_tmem = reinterpret_cast<uint32_t*>(bars + 2);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int x0 = blockIdx.x * kBX, y0 = blockIdx.y * kBY, z = blockIdx.z;

  if (tid == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc<kTmemCols>(s_tmem);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *s_tmem;

  if (tid == 0) {
    mbar_expect_tx(&bars[0], (uint32_t)(kStageB + kWeightB));
    tma_load_5d(s_in, &in_map, &bars[0], 0, x0 - 1, 0, y0 - 1, z - 1);
    bulk_load(s_w, wblob, (uint32_t)kWeightB, &bars[0]);
  }
  bool ok = tc::mbar_wait(&bars[0], 0);
  if (tid == 0 && ok) {
    tc::fence_after_sync();
    constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 16);
    const uint32_t a0 = tc::smem_u32(s_in), b0 = tc::smem_u32(s_w);
#pragma unroll 1
    for (int j = 0; j < kBY; j++) {
#pragma unroll 1
      for (int t = 0; t < 27; t++) {
        const int dx = t % 3, dy = (t / 3) % 3, dz = t / 9;  // 0..2 = offset -1..+1
        const uint32_t a = a0 + (uint32_t)((dz * kInY + j + dy) * kRowB + dx * 16);
        tc::mma_bf16(tbase + 16 * j, tc::smem_desc(a, kPlaneB, 128), tc::smem_desc(b0 + t * kTapB, 256, 128), idesc,
                     t > 0);
      }
    }
    tc::mma_commit(&bars[1]);
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, 1);
  } else {
    ok = tc::mbar_wait(&bars[1], 0);
    if (!ok && lane == 0) atomicOr(err, 2);
  }
  tc::fence_after_sync();
  if (__all_sync(0xffffffffu, ok)) {
    const int x = x0 + 32 * warp + lane;  // TMEM lane = output vertex
    const uint32_t tl = tbase + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
    for (int j = 0; j < kBY; j++) {
      float v[16];
      tc::tmem_ld16(tl + 16 * j, v);
      const int y = y0 + j;
      if (x >= D.X || y >= D.Y) continue;
      const int64_t row = (int64_t)z * D.Y + y;
      if (EPI == kEpiLogits) {
        const int64_t vid = row * D.X + x;
        out_logits[vid] = v[0] + bias[0];
        out_logits[D.N + vid] = v[1] + bias[1];
      } else {
        __nv_bfloat16* o = out_act + row * 2 * D.X * 8;  // row base, plane 0
        float m[16];
        if (EPI == kEpiMaskBf16) {
          const __nv_bfloat16* mk = mask_act + row * 2 * D.X * 8;
          const uint4 q0 = *reinterpret_cast<const uint4*>(mk + (int64_t)x * 8);
          const uint4 q1 = *reinterpret_cast<const uint4*>(mk + (int64_t)(D.X + x) * 8);
          const __nv_bfloat16* h0 = reinterpret_cast<const __nv_bfloat16*>(&q0);
          const __nv_bfloat16* h1 = reinterpret_cast<const __nv_bfloat16*>(&q1);
#pragma unroll
          for (int c = 0; c < 8; c++) {
            m[c] = __bfloat162float(h0[c]) > 0.f ? 1.f : 0.f;
            m[8 + c] = __bfloat162float(h1[c]) > 0.f ? 1.f : 0.f;
          }
        }
        __align__(16) __nv_bfloat16 r[16];
#pragma unroll
        for (int c = 0; c < 16; c++) {
          float a = v[c];
          if (EPI == kEpiReluBf16) a = fmaxf(a + bias[c], 0.f);
          else a = a * m[c];
          r[c] = __float2bfloat16_rn(a);
        }
        *reinterpret_cast<uint4*>(o + (int64_t)x * 8) = *reinterpret_cast<const uint4*>(&r[0]);
        *reinterpret_cast<uint4*>(o + (int64_t)(D.X + x) * 8) = *reinterpret_cast<const uint4*>(&r[8]);
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc<kTmemCols>(tbase);
}

// ---- tensor map of a row-planar activation ----------------------------------------------
namespace {
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}
}  // namespace

cudaError_t make_act_map(const __nv_bfloat16* act, const ConvDims& D, CUtensorMap* map) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  if ((reinterpret_cast<uintptr_t>(act) & 15u) != 0) return cudaErrorInvalidValue;
  const cuuint64_t dims[5] = {8, (cuuint64_t)D.X, 2, (cuuint64_t)D.Y, (cuuint64_t)D.Z};
  const cuuint64_t strides[4] = {16, (cuuint64_t)D.X * 16, (cuuint64_t)D.X * 32, (cuuint64_t)D.X * D.Y * 32};
  const cuuint32_t box[5] = {8, kBX + 2, 2, kInY, kInZ};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<__nv_bfloat16*>(act), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_conv3_tc(int epi, const CUtensorMap& in_map, const uint8_t* wblob, const float* bias,
                            const ConvDims& D, __nv_bfloat16* out_act, float* out_logits,
                            const __nv_bfloat16* mask_act, int* err, cudaStream_t st) {
  if ((reinterpret_cast<uintptr_t>(wblob) & 15u) != 0) return cudaErrorInvalidValue;
  const dim3 grid((unsigned)((D.X + kBX - 1) / kBX), (unsigned)((D.Y + kBY - 1) / kBY), (unsigned)D.Z);
  cudaError_t e;
  switch (epi) {
    case kEpiReluBf16:
      e = cudaFuncSetAttribute(conv3_tc_kernel<kEpiReluBf16>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemConv);
      if (e != cudaSuccess) return e;
      ::msc::count_launch();
      conv3_tc_kernel<kEpiReluBf16><<<grid, 128, kSmemConv, st>>>(in_map, wblob, bias, D, out_act, out_logits,
                                                                   mask_act, err);
      break;
    case kEpiLogits:
      e = cudaFuncSetAttribute(conv3_tc_kernel<kEpiLogits>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemConv);
      if (e != cudaSuccess) return e;
      ::msc::count_launch();
      conv3_tc_kernel<kEpiLogits><<<grid, 128, kSmemConv, st>>>(in_map, wblob, bias, D, out_act, out_logits, mask_act,
                                                                 err);
      break;
    default:
      e = cudaFuncSetAttribute(conv3_tc_kernel<kEpiMaskBf16>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemConv);
      if (e != cudaSuccess) return e;
      ::msc::count_launch();
      conv3_tc_kernel<kEpiMaskBf16><<<grid, 128, kSmemConv, st>>>(in_map, wblob, bias, D, out_act, out_logits,
                                                                   mask_act, err);
      break;
  }
  return cudaGetLastError();
}

}  // namespace msc
