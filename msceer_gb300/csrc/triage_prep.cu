// Learned triage, CUDA-core side: combinatorial steepest-path labels, input features,
// flags, and the training kernels (loss, weight gradients, Adam, weight packing).
//
// Combinatorial label of a vertex: follow the steepest discrete step (downhill for the
// ascending manifolds of minima, uphill for the descending ones) until a vertex of a
// certain terminal region, and take its region.  The step is taken over the 26
// neighbours with the drop normalised by distance -- a discrete stand-in for the
// streamline, closer to it than the 6-neighbour V-path of the lower-star gradient
// (rec_td / rec_tu, gi_extrema_region_builder.h:286-352).  Pointer jumping resolves
// the chains.
#include "label_common.cuh"
#include "triage.cuh"

namespace msc {

// ---- combinatorial labels --------------------------------------------------------------------

// Steepest discrete step over the 26 neighbours: the largest value drop per unit
// distance among the neighbours that come before v in the vertex order (after it,
// uphill), first in position order on ties.  Every step moves strictly along the
// order, so the chains are acyclic and end at an extremum or a terminal vertex.
__global__ void comb_succ_kernel(const float* __restrict__ f, const int32_t* __restrict__ lab, const VolDims V, int dir,
                                 int32_t* __restrict__ succ) {
  const int64_t N = V.X * V.Y * V.Z;
  const float inv_d[4] = {0.f, 1.f, 0.70710678f, 0.57735027f};
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    if (lab[v] >= 0) {
      succ[v] = (int32_t)v;
      continue;
    }
    const int64_t x = v % V.X, y = (v / V.X) % V.Y, z = v / (V.X * V.Y);
    const float fv = f[v];
    int64_t best = v;
    float best_slope = -1.f;
    for (int dz = -1; dz <= 1; dz++) {
      if (z + dz < 0 || z + dz >= V.Z) continue;
      for (int dy = -1; dy <= 1; dy++) {
        if (y + dy < 0 || y + dy >= V.Y) continue;
        for (int dx = -1; dx <= 1; dx++) {
          if ((dx | dy | dz) == 0 || x + dx < 0 || x + dx >= V.X) continue;
          const int64_t u = v + dx + V.X * (dy + V.Y * dz);
          if (dir < 0 ? !vgreater(f, v, u) : !vgreater(f, u, v)) continue;  // not on the way
          const float slope = (dir < 0 ? fv - f[u] : f[u] - fv) * inv_d[(dx != 0) + (dy != 0) + (dz != 0)];
          if (slope > best_slope) {
            best_slope = slope;
            best = u;
          }
        }
      }
    }
    succ[v] = (int32_t)best;
  }
}

__global__ void comb_jump_kernel(int32_t* __restrict__ succ, int64_t N, int* __restrict__ changed) {
  bool any = false;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = succ[v];
    const int32_t ss = succ[s];
    if (ss != s) {
      succ[v] = ss;
      any = true;
    }
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(changed, 1);
}

__global__ void comb_label_kernel(const int32_t* __restrict__ succ, const int32_t* __restrict__ lab, int64_t N,
                                  int32_t* __restrict__ comb) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t l = lab[succ[v]];
    comb[v] = l >= 0 ? l : kLabelNone;
  }
}

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

// Row-planar BF16 features: f standardised, |grad f| over its mean (clipped), the
// combinatorial label boundary and the certain-terminal indicator of each direction.
__global__ void features_kernel(const float* __restrict__ f, const float4* __restrict__ g,
                                const int32_t* __restrict__ comb_asc, const int32_t* __restrict__ comb_dsc,
                                const uint8_t* __restrict__ st_asc, const uint8_t* __restrict__ st_dsc, const VolDims V,
                                const double* __restrict__ sums, __nv_bfloat16* __restrict__ out) {
  const int64_t N = V.X * V.Y * V.Z;
  const double mean = sums[0] / (double)N;
  const double var = sums[1] / (double)N - mean * mean;
  const float inv_std = var > 0 ? (float)(1.0 / sqrt(var)) : 1.f;
  const float inv_g = sums[2] > 0 ? (float)((double)N / sums[2]) : 1.f;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = v % V.X, row = v / V.X;
    const float4 gv = g[v];
    float c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    c[0] = (f[v] - (float)mean) * inv_std;
    c[1] = fminf(sqrtf(gv.x * gv.x + gv.y * gv.y + gv.z * gv.z) * inv_g, 16.f);
    c[2] = label_boundary(comb_asc, V, v) ? 1.f : 0.f;
    c[3] = label_boundary(comb_dsc, V, v) ? 1.f : 0.f;
    c[4] = (st_asc[v] == kStSeed || st_asc[v] == kStTerminal) ? 1.f : 0.f;
    c[5] = (st_dsc[v] == kStSeed || st_dsc[v] == kStTerminal) ? 1.f : 0.f;
    __align__(16) __nv_bfloat16 h[8];
#pragma unroll
    for (int k = 0; k < 8; k++) h[k] = __float2bfloat16_rn(c[k]);
    __nv_bfloat16* o = out + row * 2 * V.X * 8;
    *reinterpret_cast<uint4*>(o + x * 8) = *reinterpret_cast<const uint4*>(h);
    *reinterpret_cast<uint4*>(o + (V.X + x) * 8) = make_uint4(0, 0, 0, 0);
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

// For one direction: unflagged, unaudited non-terminal vertices take their
// combinatorial label and leave the integration; the rest stay to be integrated.
// flags: bit 0 = flagged by the network, bit 1 = audit sample.
__global__ void triage_apply_kernel(const float* __restrict__ logits, float logit_threshold,
                                    const int32_t* __restrict__ comb, int32_t* __restrict__ lab,
                                    uint8_t* __restrict__ state, uint8_t* __restrict__ flags, int64_t N,
                                    uint32_t audit_q32, uint64_t audit_seed, unsigned long long* __restrict__ counts) {
  unsigned long long nf = 0, na = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    uint8_t fl = 0;
    if (state[v] == kStUnassigned) {
      const bool flagged = logits[v] > logit_threshold;
      const bool audit = !flagged && (uint32_t)(mix64(audit_seed ^ (uint64_t)v) >> 32) < audit_q32;
      fl = (flagged ? 1 : 0) | (audit ? 2 : 0);
      nf += flagged;
      na += audit;
      if (!fl) {
        lab[v] = comb[v];
        state[v] = kStAssigned;
      }
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

// audit result: sampled vertices whose integrated label differs from the combinatorial one
__global__ void audit_count_kernel(const int32_t* __restrict__ lab, const int32_t* __restrict__ comb,
                                   const uint8_t* __restrict__ flags, int64_t N, unsigned long long* __restrict__ count) {
  unsigned long long n = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x)
    n += (flags[v] == 2 && lab[v] != comb[v]);
  for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(count, n);
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

cudaError_t launch_comb_labels(const float* f, const int32_t* lab, const VolDims& V, int dir, int32_t* succ,
                               int32_t* comb, int* changed, int num_sms, cudaStream_t st) {
  const int64_t N = V.X * V.Y * V.Z;
  const int grid = num_sms * 8;
  comb_succ_kernel<<<grid, 256, 0, st>>>(f, lab, V, dir, succ);
  for (int round = 0; round < 64; round++) {
    cudaError_t e = cudaMemsetAsync(changed, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    comb_jump_kernel<<<grid, 256, 0, st>>>(succ, N, changed);
    int h = 0;
    e = cudaMemcpyAsync(&h, changed, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    if (!h) break;
  }
  comb_label_kernel<<<grid, 256, 0, st>>>(succ, lab, N, comb);
  return cudaGetLastError();
}

cudaError_t launch_features(const float* f, const float4* g, const int32_t* comb_asc, const int32_t* comb_dsc,
                            const uint8_t* st_asc, const uint8_t* st_dsc, const VolDims& V, double* sums,
                            __nv_bfloat16* out, int num_sms, cudaStream_t st) {
  const int64_t N = V.X * V.Y * V.Z;
  cudaError_t e = cudaMemsetAsync(sums, 0, 3 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  feature_stats_kernel<<<num_sms * 4, 256, 0, st>>>(f, g, N, sums);
  features_kernel<<<num_sms * 8, 256, 0, st>>>(f, g, comb_asc, comb_dsc, st_asc, st_dsc, V, sums, out);
  return cudaGetLastError();
}

cudaError_t launch_triage_apply(const float* logits, float logit_threshold, const int32_t* comb, int32_t* lab,
                                uint8_t* state, uint8_t* flags, int64_t N, float audit_frac, uint64_t audit_seed,
                                unsigned long long* counts, int num_sms, cudaStream_t st) {
  const double q = audit_frac <= 0.f ? 0.0 : (audit_frac >= 1.f ? 4294967295.0 : (double)audit_frac * 4294967296.0);
  triage_apply_kernel<<<num_sms * 8, 256, 0, st>>>(logits, logit_threshold, comb, lab, state, flags, N, (uint32_t)q,
                                                   audit_seed, counts);
  return cudaGetLastError();
}

cudaError_t launch_audit_count(const int32_t* lab, const int32_t* comb, const uint8_t* flags, int64_t N,
                               unsigned long long* count, int num_sms, cudaStream_t st) {
  audit_count_kernel<<<num_sms * 8, 256, 0, st>>>(lab, comb, flags, N, count);
  return cudaGetLastError();
}

cudaError_t launch_pack_weights(const float* params, uint8_t* blobs, cudaStream_t st) {
  pack_weights_kernel<<<(5 * 27 * 256 + 255) / 256, 256, 0, st>>>(params, blobs);
  return cudaGetLastError();
}

cudaError_t launch_bce_loss(const float* logits, const uint8_t* target, const ConvDims& D, float pos_weight,
                            float scale, __nv_bfloat16* dY, double* loss, int num_sms, cudaStream_t st) {
  bce_loss_kernel<<<num_sms * 8, 256, 0, st>>>(logits, target, D, pos_weight, scale, dY, loss);
  return cudaGetLastError();
}

cudaError_t launch_conv_wgrad(const __nv_bfloat16* X, const __nv_bfloat16* dY, const ConvDims& D, float* dW,
                              float* db, int num_sms, cudaStream_t st) {
  conv_wgrad_kernel<<<num_sms * 4, 128, 0, st>>>(X, dY, D, dW, db);
  return cudaGetLastError();
}

cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int n, float lr, int step, const uint8_t* mask,
                        cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<(n + 255) / 256, 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, 1e-8f, bc1, bc2, mask);
  return cudaGetLastError();
}

}  // namespace msc
