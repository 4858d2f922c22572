// Learned triage: shared declarations of the network kernels (triage_kernels.cu,
// triage_train.cu) and the labeling glue (msc_triage_capi.cu).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace msc {

void count_launch();  // msc_capi.cu

struct ConvDims {
  int64_t X, Y, Z, N;  // vertices per axis, N = X*Y*Z
};

enum { kEpiReluBf16 = 0, kEpiLogits = 1, kEpiMaskBf16 = 2 };

constexpr int kTriageCin = 10;  // input features of one direction (triage_prep.cu: features_kernel)
constexpr int kTriageHidden = 16;
constexpr int kTriageOut = 2;   // logit 0: P(the fix-up changes the first-pass label); logit 1 trained alike
// FP32 master parameters: W1[27][16][16] W2[27][16][16] W3[27][16][16] (cin x cout,
// unused input / output channels zero), b1[16] b2[16] b3[16]
constexpr int kTriageW = 27 * 16 * 16;
constexpr int kTriageParams = 3 * kTriageW + 3 * 16;

constexpr int kTriageBlobBytes = 5 * 27 * 512;  // forward W1..W3, input-gradient W2, W3

cudaError_t make_act_map(const __nv_bfloat16* act, const ConvDims& D, CUtensorMap* map);
cudaError_t launch_conv3_tc(int epi, const CUtensorMap& in_map, const uint8_t* wblob, const float* bias,
                            const ConvDims& D, __nv_bfloat16* out_act, float* out_logits,
                            const __nv_bfloat16* mask_act, int* err, cudaStream_t st);

struct VolDims;
cudaError_t launch_features(const float* f, const float4* g, const int32_t* lab, const uint8_t* state, const VolDims& V,
                            int dir, double* sums, __nv_bfloat16* out, int num_sms, cudaStream_t st);
cudaError_t launch_triage_apply(const float* logits, float logit_threshold, uint8_t* state, uint8_t* flags, int64_t N,
                                float audit_frac, uint64_t audit_seed, unsigned long long* counts, int num_sms,
                                cudaStream_t st);
cudaError_t launch_audit_count(const int32_t* lab, const int32_t* first, const uint8_t* flags, int64_t N,
                               unsigned long long* count, int num_sms, cudaStream_t st);
cudaError_t launch_change_targets(const int32_t* lab, const int32_t* first, int64_t N, uint8_t* targets, int num_sms,
                                  cudaStream_t st);
cudaError_t launch_pack_weights(const float* params, uint8_t* blobs, cudaStream_t st);
cudaError_t launch_bce_loss(const float* logits, const uint8_t* target, const ConvDims& D, float pos_weight,
                            float scale, __nv_bfloat16* dY, double* loss, int num_sms, cudaStream_t st);
cudaError_t launch_conv_wgrad(const __nv_bfloat16* X, const __nv_bfloat16* dY, const ConvDims& D, float* dW,
                              float* db, int num_sms, cudaStream_t st);
cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int n, float lr, int step, const uint8_t* mask,
                        cudaStream_t st);

// Host sequences (msc_triage_capi.cu).  `blobs` holds kTriageBlobBytes of packed
// weights (filled by the call); `err` is a device status word.
cudaError_t triage_forward(const __nv_bfloat16* feat, const ConvDims& D, const float* params, uint8_t* blobs,
                           __nv_bfloat16* act1, __nv_bfloat16* act2, float* logits, int* err, cudaStream_t st);

}  // namespace msc
