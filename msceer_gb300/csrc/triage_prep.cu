// Learned triage, CUDA-core side: the network's input features, the flags, and the
// training kernels (loss, weight gradients, Adam, weight packing).
//
// The triage decides which vertices the boundary fix-up re-decides.  Every vertex
// gets the cheap first-pass label (FP32, path compression); the fix-up -- re-
// integrating every vertex that has a differently labelled neighbour until it reaches
// a certain region, in waves -- costs about nine tenths of the labeling and changes
// about one label in ten.  The network predicts, per vertex, whether the fix-up would
// change its first-pass label; only flagged vertices plus a random audit sample are
// re-decided, the rest keep their first-pass label.
#include "label_common.cuh"
#include "triage.cuh"

namespace msc {

// ---- features --------------------------------------------------------------------------------

// sums of f, f^2 and |grad f| (double atomics, one per block)
__global__ void feature_stats_kernel(const float* __restrict__ f, const float4* __restrict__ g, int64_t N,
                                     double* __restrict__ sums) {
  double a = 0, b = 0, c = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    const double fv = f[v];
    const float4 gv = g[v];
    a += fv;
    b += fv * fv;
    c += sqrt((double)gv.x * gv.x + (double)gv.y * gv.y + (double)gv.z * gv.z);
  }
  __shared__ double s[3][32];
  for (int o = 16; o; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    s[0][w] = a;
    s[1][w] = b;
    s[2][w] = c;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    a = l < nw ? s[0][l] : 0;
    b = l < nw ? s[1][l] : 0;
    c = l < nw ? s[2][l] : 0;
    for (int o = 16; o; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (l == 0) {
      atomicAdd(&sums[0], a);
      atomicAdd(&sums[1], b);
      atomicAdd(&sums[2], c);
    }
  }
}

__device__ __forceinline__ bool label_boundary(const int32_t* lab, const VolDims& V, int64_t v) {
  const int64_t x = v % V.X, y = (v / V.X) % V.Y, z = v / (V.X * V.Y);
  const int32_t l = lab[v];
  bool d = false;
  if (x < V.X - 1) d |= lab[v + 1] != l;
  if (x > 0) d |= lab[v - 1] != l;
  if (y < V.Y - 1) d |= lab[v + V.X] != l;
  if (y > 0) d |= lab[v - V.X] != l;
  if (z < V.Z - 1) d |= lab[v + V.X * V.Y] != l;
  if (z > 0) d |= lab[v - V.X * V.Y] != l;
  return d;
}

// Row-planar BF16 features of one direction from its first-pass labels:
//   0  f standardised and signed so that the flow runs downhill in both directions
//   1  |grad f| over its mean (clipped)
//   2-4  the unit flow direction (-grad f / |grad f| for the ascending labels, +grad f
//        / |grad f| for the descending ones)
//   5  a 6-neighbour has another first-pass label
//   6  the certain-terminal indicator
//   7  the "reached no region" indicator
//   8  the fraction of differently labelled 6-neighbours
//   9  the vertex nearest to one voxel downstream has another first-pass label
__global__ void features_kernel(const float* __restrict__ f, const float4* __restrict__ g,
                                const int32_t* __restrict__ lab, const uint8_t* __restrict__ state, const VolDims V,
                                int dir, const double* __restrict__ sums, __nv_bfloat16* __restrict__ out) {
  const int64_t N = V.X * V.Y * V.Z;
  const double mean = sums[0] / (double)N;
  const double var = sums[1] / (double)N - mean * mean;
  const float inv_std = (var > 0 ? (float)(1.0 / sqrt(var)) : 1.f) * (dir < 0 ? 1.f : -1.f);
  const float inv_g = sums[2] > 0 ? (float)((double)N / sums[2]) : 1.f;
  const float flow = dir < 0 ? -1.f : 1.f;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = v % V.X, y = (v / V.X) % V.Y, z = v / (V.X * V.Y), row = v / V.X;
    const float4 gv = g[v];
    const int32_t l = lab[v];
    int diff = 0, nn = 0;
    const int64_t nbr[6] = {x < V.X - 1 ? v + 1 : -1, x > 0 ? v - 1 : -1, y < V.Y - 1 ? v + V.X : -1,
                            y > 0 ? v - V.X : -1, z < V.Z - 1 ? v + V.X * V.Y : -1, z > 0 ? v - V.X * V.Y : -1};
#pragma unroll
    for (int j = 0; j < 6; j++) {
      if (nbr[j] < 0) continue;
      nn++;
      diff += lab[nbr[j]] != l;
    }
    const float gm = sqrtf(gv.x * gv.x + gv.y * gv.y + gv.z * gv.z);
    const float inv_gm = gm > 0.f ? flow / gm : 0.f;
    const float ux = gv.x * inv_gm, uy = gv.y * inv_gm, uz = gv.z * inv_gm;
    auto clampi = [](float p, int64_t n) {
      int64_t q = (int64_t)floorf(p + 0.5f);
      return q < 0 ? (int64_t)0 : (q >= n ? n - 1 : q);
    };
    const int64_t d = clampi((float)x + ux, V.X) + V.X * (clampi((float)y + uy, V.Y) + V.Y * clampi((float)z + uz, V.Z));
    float c[16];
#pragma unroll
    for (int k = 0; k < 16; k++) c[k] = 0.f;
    c[0] = (f[v] - (float)mean) * inv_std;
    c[1] = fminf(gm * inv_g, 16.f);
    c[2] = ux;
    c[3] = uy;
    c[4] = uz;
    c[5] = diff > 0 ? 1.f : 0.f;
    c[6] = (state[v] == kStSeed || state[v] == kStTerminal) ? 1.f : 0.f;
    c[7] = l == kLabelNone ? 1.f : 0.f;
    c[8] = nn > 0 ? (float)diff / (float)nn : 0.f;
    c[9] = lab[d] != l ? 1.f : 0.f;
    __align__(16) __nv_bfloat16 h[16];
#pragma unroll
    for (int k = 0; k < 16; k++) h[k] = __float2bfloat16_rn(c[k]);
    __nv_bfloat16* o = out + row * 2 * V.X * 8;
    *reinterpret_cast<uint4*>(o + x * 8) = *reinterpret_cast<const uint4*>(&h[0]);
    *reinterpret_cast<uint4*>(o + (V.X + x) * 8) = *reinterpret_cast<const uint4*>(&h[8]);
  }
}

// ---- flags -----------------------------------------------------------------------------------

// splitmix64 finaliser: a fixed pseudo-random audit sample
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// For one direction: unflagged, unaudited vertices still open to the fix-up keep
// their first-pass label and leave the fix-up (state assigned); the rest stay open.
// flags: bit 0 = flagged by the network, bit 1 = audit sample.
__global__ void triage_apply_kernel(const float* __restrict__ logits, float logit_threshold, uint8_t* __restrict__ state,
                                    uint8_t* __restrict__ flags, int64_t N, uint32_t audit_q32, uint64_t audit_seed,
                                    unsigned long long* __restrict__ counts) {
  unsigned long long nf = 0, na = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    uint8_t fl = 0;
    if (state[v] == kStUnassigned) {
      const bool flagged = logits[v] > logit_threshold;
      const bool audit = !flagged && (uint32_t)(mix64(audit_seed ^ (uint64_t)v) >> 32) < audit_q32;
      fl = (flagged ? 1 : 0) | (audit ? 2 : 0);
      nf += flagged;
      na += audit;
      if (!fl) state[v] = kStAssigned;
    }
    flags[v] = fl;
  }
  for (int o = 16; o; o >>= 1) {
    nf += __shfl_xor_sync(0xffffffffu, nf, o);
    na += __shfl_xor_sync(0xffffffffu, na, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&counts[0], nf);
    atomicAdd(&counts[1], na);
  }
}

// audit result: sampled (unflagged) vertices whose label the fix-up changed
__global__ void audit_count_kernel(const int32_t* __restrict__ lab, const int32_t* __restrict__ first,
                                   const uint8_t* __restrict__ flags, int64_t N, unsigned long long* __restrict__ count) {
  unsigned long long n = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x)
    n += (flags[v] == 2 && lab[v] != first[v]);
  for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(count, n);
}

// training targets: 1 where the fix-up changed the first-pass label (both output rows)
__global__ void change_targets_kernel(const int32_t* __restrict__ lab, const int32_t* __restrict__ first, int64_t N,
                                      uint8_t* __restrict__ targets) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t y = lab[v] != first[v];
    targets[v] = y;
    targets[N + v] = y;
  }
}

// ---- weights ---------------------------------------------------------------------------------

// FP32 master weights W[l][tap][cin][cout] -> BF16 MMA operand blobs: forward (B[n=cout][k=cin])
// for the three layers, then the input-gradient blobs of layers 2 and 3 (taps mirrored,
// B[n=cin][k=cout]).
__global__ void pack_weights_kernel(const float* __restrict__ params, uint8_t* __restrict__ blobs) {
  const int total = 5 * 27 * 256;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int b = i / (27 * 256), r = i % (27 * 256);
    const int t = r / 256, n = (r / 16) % 16, k = r % 16;
    float w;
    if (b < 3) {
      w = params[b * kTriageW + t * 256 + k * 16 + n];  // cin = k, cout = n
    } else {
      const int l = b - 2;  // layer 2 or 3 (0-based 1, 2)
      w = params[l * kTriageW + (26 - t) * 256 + n * 16 + k];  // cin = n, cout = k
    }
    __nv_bfloat16* dst = reinterpret_cast<__nv_bfloat16*>(blobs + (size_t)b * 27 * 512 + t * 512 + (k / 8) * 256 + n * 16);
    dst[k % 8] = __float2bfloat16_rn(w);
  }
}

// ---- training --------------------------------------------------------------------------------

// Weighted binary cross-entropy on both outputs.  Writes the logit gradients as a
// row-planar BF16 tensor (channels 0, 1) and accumulates the loss.
__global__ void bce_loss_kernel(const float* __restrict__ logits, const uint8_t* __restrict__ target, const ConvDims D,
                                float pos_weight, float scale, __nv_bfloat16* __restrict__ dY, double* __restrict__ loss) {
  double acc = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < D.N; v += (int64_t)gridDim.x * blockDim.x) {
    float gz[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const float z = logits[c * D.N + v];
      const float y = target[c * D.N + v] ? 1.f : 0.f;
      const float w = y > 0.f ? pos_weight : 1.f;
      const float sp = fmaxf(z, 0.f) + log1pf(expf(-fabsf(z)));  // softplus(z)
      acc += (double)(w * (sp - y * z) * scale);
      const float sg = 1.f / (1.f + expf(-z));
      gz[c] = w * (sg - y) * scale;
    }
    const int64_t x = v % D.X, row = v / D.X;
    __align__(16) __nv_bfloat16 h[8];
    h[0] = __float2bfloat16_rn(gz[0]);
    h[1] = __float2bfloat16_rn(gz[1]);
#pragma unroll
    for (int k = 2; k < 8; k++) h[k] = __float2bfloat16_rn(0.f);
    __nv_bfloat16* o = dY + row * 2 * D.X * 8;
    *reinterpret_cast<uint4*>(o + x * 8) = *reinterpret_cast<const uint4*>(h);
    *reinterpret_cast<uint4*>(o + (D.X + x) * 8) = make_uint4(0, 0, 0, 0);
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// dW[tap][cin][cout] += sum_v X[v + tap][cin] * dY[v][cout] and db[cout] += sum_v dY[v][cout]
// over a block of 32 (x) x 4 (y) output vertices at one z.  Thread (cin, cout pair)
// keeps 27 x 2 accumulators; X (with its halo) and dY are staged as FP32.
constexpr int kGWX = 32, kGWY = 4;
__global__ void __launch_bounds__(128) conv_wgrad_kernel(const __nv_bfloat16* __restrict__ X,
                                                         const __nv_bfloat16* __restrict__ dY, const ConvDims D,
                                                         float* __restrict__ dW, float* __restrict__ db) {
  __shared__ float sx[3][kGWY + 2][kGWX + 2][16];
  __shared__ float sy[kGWY][kGWX][16];
  const int tid = threadIdx.x;
  const int cin = tid >> 3, cp = (tid & 7) * 2;
  float acc[27][2];
#pragma unroll
  for (int t = 0; t < 27; t++) acc[t][0] = acc[t][1] = 0.f;
  float bacc[2] = {0.f, 0.f};
  const int64_t ntx = (D.X + kGWX - 1) / kGWX, nty = (D.Y + kGWY - 1) / kGWY;
  const int64_t nblk = ntx * nty * D.Z;
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t bx = blk % ntx, by = (blk / ntx) % nty, bz = blk / (ntx * nty);
    const int64_t x0 = bx * kGWX, y0 = by * kGWY;
    __syncthreads();
    // X with a one-vertex halo (zero outside), 16 channels
    for (int i = tid; i < 3 * (kGWY + 2) * (kGWX + 2) * 2; i += 128) {
      const int half = i & 1, p = i >> 1;
      const int lx = p % (kGWX + 2), ly = (p / (kGWX + 2)) % (kGWY + 2), lz = p / ((kGWX + 2) * (kGWY + 2));
      const int64_t gx = x0 + lx - 1, gy = y0 + ly - 1, gz = bz + lz - 1;
      float* dst = &sx[lz][ly][lx][half * 8];
      if (gx < 0 || gy < 0 || gz < 0 || gx >= D.X || gy >= D.Y || gz >= D.Z) {
#pragma unroll
        for (int c = 0; c < 8; c++) dst[c] = 0.f;
      } else {
        const uint4 q = *reinterpret_cast<const uint4*>(X + ((gz * D.Y + gy) * 2 + half) * D.X * 8 + gx * 8);
        const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
        for (int c = 0; c < 8; c++) dst[c] = __bfloat162float(h[c]);
      }
    }
    for (int i = tid; i < kGWY * kGWX * 2; i += 128) {
      const int half = i & 1, p = i >> 1;
      const int lx = p % kGWX, ly = p / kGWX;
      const int64_t gx = x0 + lx, gy = y0 + ly;
      float* dst = &sy[ly][lx][half * 8];
      if (gx >= D.X || gy >= D.Y) {
#pragma unroll
        for (int c = 0; c < 8; c++) dst[c] = 0.f;
      } else {
        const uint4 q = *reinterpret_cast<const uint4*>(dY + ((bz * D.Y + gy) * 2 + half) * D.X * 8 + gx * 8);
        const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
        for (int c = 0; c < 8; c++) dst[c] = __bfloat162float(h[c]);
      }
    }
    __syncthreads();
#pragma unroll 1
    for (int ly = 0; ly < kGWY; ly++) {
#pragma unroll 1
      for (int lx = 0; lx < kGWX; lx++) {
        const float g0 = sy[ly][lx][cp], g1 = sy[ly][lx][cp + 1];
        bacc[0] += g0;
        bacc[1] += g1;
#pragma unroll
        for (int t = 0; t < 27; t++) {
          const float xv = sx[t / 9][ly + (t / 3) % 3][lx + t % 3][cin];
          acc[t][0] = fmaf(xv, g0, acc[t][0]);
          acc[t][1] = fmaf(xv, g1, acc[t][1]);
        }
      }
    }
  }
#pragma unroll
  for (int t = 0; t < 27; t++) {
    atomicAdd(&dW[t * 256 + cin * 16 + cp], acc[t][0]);
    atomicAdd(&dW[t * 256 + cin * 16 + cp + 1], acc[t][1]);
  }
  if (cin == 0) {
    atomicAdd(&db[cp], bacc[0]);
    atomicAdd(&db[cp + 1], bacc[1]);
  }
}

// Adam on the FP32 master parameters; `mask` zeroes the padded channels' updates.
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float bc1, float bc2,
                            const uint8_t* __restrict__ mask) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!mask[i]) {
      p[i] = 0.f;
      continue;
    }
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// ---- launchers -------------------------------------------------------------------------------

cudaError_t launch_features(const float* f, const float4* g, const int32_t* lab, const uint8_t* state, const VolDims& V,
                            int dir, double* sums, __nv_bfloat16* out, int num_sms, cudaStream_t st) {
  const int64_t N = V.X * V.Y * V.Z;
  cudaError_t e = cudaMemsetAsync(sums, 0, 3 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  ::msc::count_launch();
  feature_stats_kernel<<<num_sms * 4, 256, 0, st>>>(f, g, N, sums);
  ::msc::count_launch();
  features_kernel<<<num_sms * 8, 256, 0, st>>>(f, g, lab, state, V, dir, sums, out);
  return cudaGetLastError();
}

cudaError_t launch_triage_apply(const float* logits, float logit_threshold, uint8_t* state, uint8_t* flags, int64_t N,
                                float audit_frac, uint64_t audit_seed, unsigned long long* counts, int num_sms,
                                cudaStream_t st) {
  const double q = audit_frac <= 0.f ? 0.0 : (audit_frac >= 1.f ? 4294967295.0 : (double)audit_frac * 4294967296.0);
  ::msc::count_launch();
  triage_apply_kernel<<<num_sms * 8, 256, 0, st>>>(logits, logit_threshold, state, flags, N, (uint32_t)q, audit_seed,
                                                   counts);
  return cudaGetLastError();
}

cudaError_t launch_audit_count(const int32_t* lab, const int32_t* first, const uint8_t* flags, int64_t N,
                               unsigned long long* count, int num_sms, cudaStream_t st) {
  ::msc::count_launch();
  audit_count_kernel<<<num_sms * 8, 256, 0, st>>>(lab, first, flags, N, count);
  return cudaGetLastError();
}

cudaError_t launch_change_targets(const int32_t* lab, const int32_t* first, int64_t N, uint8_t* targets, int num_sms,
                                  cudaStream_t st) {
  ::msc::count_launch();
  change_targets_kernel<<<num_sms * 8, 256, 0, st>>>(lab, first, N, targets);
  return cudaGetLastError();
}

cudaError_t launch_pack_weights(const float* params, uint8_t* blobs, cudaStream_t st) {
  ::msc::count_launch();
  pack_weights_kernel<<<(5 * 27 * 256 + 255) / 256, 256, 0, st>>>(params, blobs);
  return cudaGetLastError();
}

cudaError_t launch_bce_loss(const float* logits, const uint8_t* target, const ConvDims& D, float pos_weight,
                            float scale, __nv_bfloat16* dY, double* loss, int num_sms, cudaStream_t st) {
  ::msc::count_launch();
  bce_loss_kernel<<<num_sms * 8, 256, 0, st>>>(logits, target, D, pos_weight, scale, dY, loss);
  return cudaGetLastError();
}

cudaError_t launch_conv_wgrad(const __nv_bfloat16* X, const __nv_bfloat16* dY, const ConvDims& D, float* dW,
                              float* db, int num_sms, cudaStream_t st) {
  ::msc::count_launch();
  conv_wgrad_kernel<<<num_sms * 4, 128, 0, st>>>(X, dY, D, dW, db);
  return cudaGetLastError();
}

cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int n, float lr, int step, const uint8_t* mask,
                        cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  ::msc::count_launch();
  adam_kernel<<<(n + 255) / 256, 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, 1e-8f, bc1, bc2, mask);
  return cudaGetLastError();
}

}  // namespace msc
