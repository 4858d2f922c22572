// extern "C" entry points of the triage network (include/msc_triage.h): forward,
// backward and the optimiser step, as host sequences of the kernels in
// triage_kernels.cu (tensor-core convolutions) and triage_prep.cu.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/msc_triage.h"
#include "triage.cuh"

namespace msc {

cudaError_t triage_forward(const __nv_bfloat16* feat, const ConvDims& D, const float* params, uint8_t* blobs,
                           __nv_bfloat16* act1, __nv_bfloat16* act2, float* logits, int* err, cudaStream_t st) {
  cudaError_t e = launch_pack_weights(params, blobs, st);
  if (e != cudaSuccess) return e;
  CUtensorMap m0, m1, m2;
  if ((e = make_act_map(feat, D, &m0)) != cudaSuccess) return e;
  if ((e = make_act_map(act1, D, &m1)) != cudaSuccess) return e;
  if ((e = make_act_map(act2, D, &m2)) != cudaSuccess) return e;
  const float* bias = params + 3 * kTriageW;
  if ((e = launch_conv3_tc(kEpiReluBf16, m0, blobs, bias, D, act1, nullptr, nullptr, err, st)) != cudaSuccess) return e;
  if ((e = launch_conv3_tc(kEpiReluBf16, m1, blobs + 27 * 512, bias + 16, D, act2, nullptr, nullptr, err, st)) !=
      cudaSuccess)
    return e;
  return launch_conv3_tc(kEpiLogits, m2, blobs + 2 * 27 * 512, bias + 32, D, nullptr, logits, nullptr, err, st);
}

}  // namespace msc

namespace {

thread_local std::string t_err;

int fail(int code, const std::string& m) {
  t_err = m;
  return code;
}

#define TCUDA(expr, what)                                                                     \
  do {                                                                                        \
    cudaError_t e_ = (expr);                                                                  \
    if (e_ != cudaSuccess) return fail(MSC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

bool conv_dims(const int64_t* dims, msc::ConvDims* D) {
  if (!dims || dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return false;
  if (dims[0] > (1 << 24) || dims[1] > (1 << 24) || dims[2] > 65535) return false;
  *D = msc::ConvDims{dims[0], dims[1], dims[2], dims[0] * dims[1] * dims[2]};
  return true;
}

// device scratch of one call, freed in stream order
struct Scratch {
  cudaStream_t st;
  std::vector<void*> p;
  explicit Scratch(cudaStream_t s) : st(s) {}
  ~Scratch() {
    for (void* q : p) cudaFreeAsync(q, st);
  }
  template <class T>
  cudaError_t get(T** out, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, bytes, st);
    if (e == cudaSuccess) {
      p.push_back(q);
      *out = reinterpret_cast<T*>(q);
    }
    return e;
  }
};

int read_err(const int* d, cudaStream_t st) {
  int h = 0;
  TCUDA(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, st), "read status");
  TCUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (h) return fail(MSC_ERR_CUDA, "tensor-core pipeline wait timed out");
  return MSC_OK;
}

// trainable entries: layer 1 input channels < 6, layer 3 output channels < 2
std::vector<uint8_t> param_mask() {
  std::vector<uint8_t> m(MSC_TRIAGE_PARAMS, 1);
  for (int t = 0; t < 27; t++)
    for (int ci = 0; ci < 16; ci++)
      for (int co = 0; co < 16; co++) {
        if (ci >= msc::kTriageCin) m[0 * msc::kTriageW + t * 256 + ci * 16 + co] = 0;
        if (co >= msc::kTriageOut) m[2 * msc::kTriageW + t * 256 + ci * 16 + co] = 0;
      }
  for (int co = msc::kTriageOut; co < 16; co++) m[3 * msc::kTriageW + 32 + co] = 0;
  return m;
}

}  // namespace

extern "C" {

const char* msc_triage_last_error_string(void) { return t_err.c_str(); }

int msc_triage_forward_3d(const uint16_t* features, const int64_t dims[3], const float* weights, uint16_t* act1,
                          uint16_t* act2, float* logits, msc_stream_t stream) {
  msc::ConvDims D;
  if (!conv_dims(dims, &D)) return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  if (!features || !weights || !logits) return fail(MSC_ERR_NULL_POINTER, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  Scratch s(st);
  uint8_t* blobs;
  int* err;
  __nv_bfloat16 *a1 = reinterpret_cast<__nv_bfloat16*>(act1), *a2 = reinterpret_cast<__nv_bfloat16*>(act2);
  TCUDA(s.get(&blobs, msc::kTriageBlobBytes), "alloc");
  TCUDA(s.get(&err, sizeof(int)), "alloc");
  TCUDA(cudaMemsetAsync(err, 0, sizeof(int), st), "memset");
  if (!a1) TCUDA(s.get(&a1, (size_t)D.N * 32), "alloc");
  if (!a2) TCUDA(s.get(&a2, (size_t)D.N * 32), "alloc");
  TCUDA(msc::triage_forward(reinterpret_cast<const __nv_bfloat16*>(features), D, weights, blobs, a1, a2, logits, err,
                            st),
        "triage forward");
  return read_err(err, st);
}

int msc_triage_backward_3d(const uint16_t* features, const uint16_t* act1, const uint16_t* act2, const float* logits,
                           const uint8_t* targets, const int64_t dims[3], const float* weights, float pos_weight,
                           float* grads, double* loss, msc_stream_t stream) {
  msc::ConvDims D;
  if (!conv_dims(dims, &D)) return fail(MSC_ERR_BAD_DIMS, "invalid dims");
  if (!features || !act1 || !act2 || !logits || !targets || !weights || !grads || !loss)
    return fail(MSC_ERR_NULL_POINTER, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int sms = sm_count();
  Scratch s(st);
  uint8_t* blobs;
  int* err;
  __nv_bfloat16 *dy3, *dy2, *dy1;
  TCUDA(s.get(&blobs, msc::kTriageBlobBytes), "alloc");
  TCUDA(s.get(&err, sizeof(int)), "alloc");
  TCUDA(s.get(&dy3, (size_t)D.N * 32), "alloc");
  TCUDA(s.get(&dy2, (size_t)D.N * 32), "alloc");
  TCUDA(s.get(&dy1, (size_t)D.N * 32), "alloc");
  TCUDA(cudaMemsetAsync(err, 0, sizeof(int), st), "memset");
  TCUDA(cudaMemsetAsync(grads, 0, MSC_TRIAGE_PARAMS * sizeof(float), st), "memset");
  TCUDA(cudaMemsetAsync(loss, 0, sizeof(double), st), "memset");
  TCUDA(msc::launch_pack_weights(weights, blobs, st), "pack weights");
  const auto* feat = reinterpret_cast<const __nv_bfloat16*>(features);
  const auto* a1 = reinterpret_cast<const __nv_bfloat16*>(act1);
  const auto* a2 = reinterpret_cast<const __nv_bfloat16*>(act2);
  const float scale = 1.f / (float)(2 * D.N);
  TCUDA(msc::launch_bce_loss(logits, targets, D, pos_weight, scale, dy3, loss, sms, st), "loss");
  float* gW = grads;
  float* gb = grads + 3 * msc::kTriageW;
  // layer 3
  TCUDA(msc::launch_conv_wgrad(a2, dy3, D, gW + 2 * msc::kTriageW, gb + 32, sms, st), "weight gradient 3");
  CUtensorMap m3, m2;
  TCUDA(msc::make_act_map(dy3, D, &m3), "tensor map");
  TCUDA(msc::launch_conv3_tc(msc::kEpiMaskBf16, m3, blobs + 4 * 27 * 512, nullptr, D, dy2, nullptr, a2, err, st),
        "input gradient 3");
  // layer 2
  TCUDA(msc::launch_conv_wgrad(a1, dy2, D, gW + msc::kTriageW, gb + 16, sms, st), "weight gradient 2");
  TCUDA(msc::make_act_map(dy2, D, &m2), "tensor map");
  TCUDA(msc::launch_conv3_tc(msc::kEpiMaskBf16, m2, blobs + 3 * 27 * 512, nullptr, D, dy1, nullptr, a1, err, st),
        "input gradient 2");
  // layer 1
  TCUDA(msc::launch_conv_wgrad(feat, dy1, D, gW, gb, sms, st), "weight gradient 1");
  return read_err(err, st);
}

int msc_triage_adam_step(float* weights, const float* grads, float* m, float* v, int step, float lr,
                         msc_stream_t stream) {
  if (!weights || !grads || !m || !v) return fail(MSC_ERR_NULL_POINTER, "null argument");
  if (step < 1) return fail(MSC_ERR_BAD_DIMS, "step counts from 1");
  cudaStream_t st = (cudaStream_t)stream;
  static const std::vector<uint8_t> mask_h = param_mask();
  Scratch s(st);
  uint8_t* mask;
  TCUDA(s.get(&mask, mask_h.size()), "alloc");
  TCUDA(cudaMemcpyAsync(mask, mask_h.data(), mask_h.size(), cudaMemcpyHostToDevice, st), "copy mask");
  TCUDA(msc::launch_adam(weights, grads, m, v, MSC_TRIAGE_PARAMS, lr, step, mask, st), "adam");
  TCUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  return MSC_OK;
}

}  // extern "C"
