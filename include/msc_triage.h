/* Learned triage for the integrated labels of libmsc_gpu.so.
 *
 * No counterpart in the reference: MSCEER integrates every vertex.  A small 3D
 * convolutional network (three 3x3x3 layers, 6 -> 16 -> 16 -> 2 channels, BF16
 * weights and activations with FP32 accumulation on the tensor cores) predicts, per
 * vertex and direction, whether the integrated destination differs from the
 * combinatorial steepest-path destination.  Only flagged vertices plus a random audit
 * sample are integrated; the others take the combinatorial label.  The plain path
 * (msc_integrated_labels_3d) stays the drop-in and the judge of the triage's mismatch.
 *
 * Tensors:
 *   features / activations   BF16, "row-planar" [Z][Y][2][X][8] (16 channels per
 *                            vertex, channels 0-7 then 8-15 of each row), X*Y*Z*32 bytes
 *   logits                   FP32 [2][X*Y*Z]: ascending then descending
 *   targets                  uint8 [2][X*Y*Z]: 1 where the label differs
 *   weights                  FP32 [MSC_TRIAGE_PARAMS]: W1, W2, W3 as [27 taps][16 cin][16 cout]
 *                            (tap = dx + 3 dy + 9 dz, offsets -1..1), then b1, b2, b3 [16];
 *                            channels beyond 6 inputs / 2 outputs must be zero
 * All pointers are device memory; every call runs on `stream`, synchronises it, and
 * returns MSC_OK or a negative MSC_ERR_* code (text: msc_triage_last_error_string()
 * for the network entries, msc_labels_last_error_string() for the labeling ones). */
#ifndef MSC_TRIAGE_H
#define MSC_TRIAGE_H

#include <stdint.h>

#include "msc_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MSC_TRIAGE_IN_CHANNELS 6
#define MSC_TRIAGE_OUT_CHANNELS 2
#define MSC_TRIAGE_PARAMS (3 * 27 * 16 * 16 + 3 * 16)

typedef struct {
  const float* weights;        /* device, MSC_TRIAGE_PARAMS floats */
  float logit_threshold_asc;   /* integrate a vertex whose logit exceeds the threshold */
  float logit_threshold_dsc;
  float audit_fraction;        /* additionally integrate this random fraction of the rest */
  uint64_t audit_seed;
} msc_triage_params;

/* Network inputs of a volume: runs the labeling chain up to the certain terminal
 * regions of both directions, the combinatorial labels (comb: int32 [2][X*Y*Z],
 * -1 = none) and the features. */
int msc_triage_features_3d(const float* f, const uint8_t* grad, const int64_t dims[3], const msc_integ_params* params,
                           uint16_t* features, int32_t* comb, msc_stream_t stream);

/* Error text of the last failed network call on the calling thread. */
const char* msc_triage_last_error_string(void);

/* Forward pass: act1, act2 (row-planar BF16, may be NULL only together with a
 * non-training use) and logits. */
int msc_triage_forward_3d(const uint16_t* features, const int64_t dims[3], const float* weights, uint16_t* act1,
                          uint16_t* act2, float* logits, msc_stream_t stream);

/* Weighted binary cross-entropy (positives weighted by pos_weight, mean over 2*X*Y*Z
 * outputs) and its gradient with respect to every parameter (grads: FP32
 * [MSC_TRIAGE_PARAMS], overwritten); loss (device double) receives the loss. */
int msc_triage_backward_3d(const uint16_t* features, const uint16_t* act1, const uint16_t* act2, const float* logits,
                           const uint8_t* targets, const int64_t dims[3], const float* weights, float pos_weight,
                           float* grads, double* loss, msc_stream_t stream);

/* One Adam step (beta 0.9 / 0.999) on weights with moment buffers m, v (FP32
 * [MSC_TRIAGE_PARAMS]); step counts from 1.  Padded channels stay zero. */
int msc_triage_adam_step(float* weights, const float* grads, float* m, float* v, int step, float lr,
                         msc_stream_t stream);

/* Integrated labels with triage: as msc_integrated_labels_3d, integrating only
 * flagged and audited vertices.  stats (host, optional) receives per direction
 * (ascending, then descending): flagged, audited, audited whose integrated label
 * differs from the combinatorial one, boundary re-decisions. */
int msc_triage_labels_3d(const float* f, const uint8_t* grad, const int64_t dims[3], const msc_integ_params* params,
                         const msc_triage_params* triage, int32_t* labels_asc, int32_t* labels_dsc, int64_t stats[8],
                         msc_stream_t stream);

/* The whole ondemandaccurate labeling from host memory, for hosts without device
 * buffers: copies f (X*Y*Z floats) to the device, computes the lower-star .grad and
 * the ascending and descending labels -- with triage when `triage` is not NULL
 * (its weights stay a device pointer), plain full integration otherwise -- and copies
 * the labels back (X*Y*Z int32 each).  Replaces the compute of ondemandaccurate.cxx
 * between loading the image and writing the labels.  Blocking. */
int msc_ondemand_labels_host(const float* f, const int64_t dims[3], const msc_integ_params* params,
                             const msc_triage_params* triage, int32_t* labels_asc, int32_t* labels_dsc);

#ifdef __cplusplus
}
#endif

#endif /* MSC_TRIAGE_H */
