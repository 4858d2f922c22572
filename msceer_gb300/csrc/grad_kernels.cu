// K3: central-difference gradient of the image, sm_103a.
//
// Replaces RegularGridTrilinearFunction::ComputeGradFromImage(1)
// (gi_regular_grid_trilinear_function.h:328-341) / GradientFromImage (:285-307):
// per axis, sum_i kRKCoefficients[k][i] * f(neighbour i) with k = 1 inside
// (coefficients -1/2, 0, 1/2; src/gi_regular_grid_trilinear_function.cxx:5-11) and
// k = 0 on a first or last plane (Gather1DNeighborhood shrinks the kernel to the
// distance to the boundary, gi_regular_grid.h:270-303), i.e. the component is 0 there.
//
// The reference forms each product in float and accumulates in double.  The f64
// variant reproduces that exactly; the f32 variants round 0.5*(f[+1] - f[-1]) once
// to float (within half an ulp of the f64 value).  One thread per vertex, x fastest;
// neighbour loads hit L1 (the x-neighbours are shared by the warp) and the outputs
// are stored as one 16-byte vector per vertex in the padded layout.
#include "msc_device.cuh"

namespace msc {

template <int ND, int LAYOUT>  // LAYOUT: 0 = xyz f32 (ND floats), 1 = xyzw f32, 2 = xyz f64
__global__ void __launch_bounds__(256) central_diff_kernel(const float* __restrict__ f, void* __restrict__ out,
                                                           const int64_t X, const int64_t Y, const int64_t Z) {
  const int64_t n = X * Y * Z;
  const bool small = n <= (int64_t)0xFFFFFFFF;  // 32-bit index arithmetic (64-bit division is slow)
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    int64_t x, y, z;
    if (small) {
      const uint32_t u = (uint32_t)v, r = u / (uint32_t)X;
      x = u - r * (uint32_t)X;
      y = r % (uint32_t)Y;
      z = r / (uint32_t)Y;
    } else {
      const int64_t r = v / X;
      x = v - r * X;
      y = r % Y;
      z = r / Y;
    }
    const bool ix = x > 0 && x < X - 1;
    const bool iy = y > 0 && y < Y - 1;
    const bool iz = (ND == 3) && z > 0 && z < Z - 1;
    const float* p = f + v;
    float ax = 0.f, bx = 0.f, ay = 0.f, by = 0.f, az = 0.f, bz = 0.f;
    if (ix) { ax = __ldg(p - 1); bx = __ldg(p + 1); }
    if (iy) { ay = __ldg(p - X); by = __ldg(p + X); }
    if (iz) { az = __ldg(p - X * Y); bz = __ldg(p + X * Y); }
    if constexpr (LAYOUT == 2) {
      const float c = __ldg(p);
      // res = 0 + (-0.5f*a) + (0.0f*c) + (0.5f*b), each product a float, summed in double
      auto comp = [&](bool inside, float a, float b) -> double {
        if (!inside) return 0.0 + (double)(0.0f * c);
        double s = 0.0;
        s += (double)(-0.5f * a);
        s += (double)(0.0f * c);
        s += (double)(0.5f * b);
        return s;
      };
      double* o = reinterpret_cast<double*>(out) + v * ND;
      o[0] = comp(ix, ax, bx);
      o[1] = comp(iy, ay, by);
      if (ND == 3) o[2] = comp(iz, az, bz);
    } else {
      const float gx = ix ? 0.5f * (bx - ax) : 0.f;
      const float gy = iy ? 0.5f * (by - ay) : 0.f;
      const float gz = iz ? 0.5f * (bz - az) : 0.f;
      if constexpr (LAYOUT == 1) {
        if (ND == 3)
          reinterpret_cast<float4*>(out)[v] = make_float4(gx, gy, gz, 0.f);
        else
          reinterpret_cast<float2*>(out)[v] = make_float2(gx, gy);
      } else {
        float* o = reinterpret_cast<float*>(out) + v * ND;
        o[0] = gx;
        o[1] = gy;
        if (ND == 3) o[2] = gz;
      }
    }
  }
}

cudaError_t launch_central_diff(int nd, int layout, const float* f, void* out, const GradDims& D, int num_sms,
                                cudaStream_t stream) {
  const int64_t n = D.v[0] * D.v[1] * D.v[2];
  const int64_t blocks = (n + 255) / 256;
  const int64_t cap = (int64_t)num_sms * 8;
  const int grid = (int)(blocks < cap ? blocks : cap);
  if (grid <= 0) return cudaSuccess;
  const int64_t X = D.v[0], Y = D.v[1], Z = D.v[2];
#define MSC_LAUNCH(ND_, L_) (count_launch(), central_diff_kernel<ND_, L_><<<grid, 256, 0, stream>>>(f, out, X, Y, Z))
  if (nd == 3) {
    if (layout == 0) MSC_LAUNCH(3, 0);
    else if (layout == 1) MSC_LAUNCH(3, 1);
    else MSC_LAUNCH(3, 2);
  } else {
    if (layout == 0) MSC_LAUNCH(2, 0);
    else if (layout == 1) MSC_LAUNCH(2, 1);
    else MSC_LAUNCH(2, 2);
  }
#undef MSC_LAUNCH
  return cudaGetLastError();
}

}  // namespace msc
