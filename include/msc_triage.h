/* Learned triage for the integrated labels of libmsc_gpu.so.
 *
 * No counterpart in the reference: MSCEER re-decides every vertex next to a label
 * boundary.  The labeling has a cheap first pass (FP32 streamlines with path
 * compression) and an expensive boundary fix-up (every vertex with a differently
 * labelled 6-neighbour re-integrated until it reaches a certain region, in waves),
 * which takes about nine tenths of the time and changes about one first-pass label in
 * ten.  A small 3D convolutional network (three 3x3x3 layers, 6 -> 16 -> 16 -> 2
 * channels, BF16 weights and activations with FP32 accumulation on the tensor cores)
 * predicts, per vertex, whether the fix-up would change its first-pass label; only
 * flagged vertices plus a random audit sample are re-decided, the rest keep the
 * first-pass label.  The plain path (msc_integrated_labels_3d) stays the drop-in and
 * the yardstick of the triage's mismatch.  One network serves both directions: the
 * features of the descending direction see -f.
 *
 * Tensors:
 *   features / activations   BF16, "row-planar" [Z][Y][2][X][8] (16 channels per
 *                            vertex, channels 0-7 then 8-15 of each row), X*Y*Z*32 bytes
 *   logits                   FP32 [2][X*Y*Z]; channel 0 decides, channel 1 is trained alike
 *   targets                  uint8 [2][X*Y*Z]: 1 where the fix-up changes the label (both rows)
 *   weights                  FP32 [MSC_TRIAGE_PARAMS]: W1, W2, W3 as [27 taps][16 cin][16 cout]
 *                            (tap = dx + 3 dy + 9 dz, offsets -1..1), then b1, b2, b3 [16];
 *                            channels beyond 10 inputs / 2 outputs must be zero
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

#define MSC_TRIAGE_IN_CHANNELS 10
#define MSC_TRIAGE_OUT_CHANNELS 2
#define MSC_TRIAGE_PARAMS (3 * 27 * 16 * 16 + 3 * 16)

typedef struct {
  const float* weights;        /* device, MSC_TRIAGE_PARAMS floats */
  float logit_threshold_asc;   /* integrate a vertex whose logit exceeds the threshold */
  float logit_threshold_dsc;
  float audit_fraction;        /* additionally integrate this random fraction of the rest */
  uint64_t audit_seed;
} msc_triage_params;

/* Training data of a volume: for the ascending then the descending direction, the
 * network features after the first pass (features: 2 row-planar tensors, 2*X*Y*Z*32
 * bytes) and, when `targets` is not NULL, the targets of the full fix-up (uint8
 * [2 directions][2][X*Y*Z]). */
int msc_triage_features_3d(const float* f, const uint8_t* grad, const int64_t dims[3], const msc_integ_params* params,
                           uint16_t* features, uint8_t* targets, msc_stream_t stream);

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

/* Integrated labels with triage: as msc_integrated_labels_3d, with the boundary
 * fix-up restricted to flagged and audited vertices.  stats (host, optional)
 * receives per direction (ascending, then descending): flagged, audited, audited
 * whose label the fix-up changed (the misses the network would have made there),
 * boundary re-decisions. */
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
