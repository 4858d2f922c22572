// Conforming gradient of ondemandaccurate's accurate 3-manifolds (sm_103a).
//
// Replaces, with identical output bytes:
//   VertexLabelingToBoundaryLabeling::ComputeMINBoundary / ComputeMAXBoundary
//     (gi_labeling_to_bounary_labeling.h:48-199): one restriction byte per cell from the
//     final ascending / descending labels
//   the re-pairing loop of ondemandaccurate.cxx:1000-1063 with
//     MyRobinsNoalloc<...,4,6>::ComputeLowerStar (gi_modified_robins.h:1281-1343): the
//     touched vertices' lower stars recomputed, split by restriction label
// The ascending-manifold closure of RecordGrad (:693-699) runs afterwards as the ldir
// stage of the .grad (ldir_kernels.cu) from the roots written here.
//
// The restriction passes run one launch per cell dimension, since each reads the bytes
// the previous one wrote (the reference separates them by barriers); every thread owns
// one cell and only writes it.
#include "lstar_core.cuh"
#include "msc_device.cuh"

namespace msc {

namespace {

__device__ __forceinline__ void cell_xyz(const GradDims& D, int64_t id, int64_t c[3]) {
  if ((uint64_t)id <= 0xFFFFFFFFull && D.d[0] * D.d[1] <= 0xFFFFFFFFll) {
    const uint32_t u = (uint32_t)id, dx = (uint32_t)D.d[0], dy = (uint32_t)D.d[1];
    const uint32_t q = u / dx;
    c[0] = u - q * dx;
    c[1] = q % dy;
    c[2] = q / dy;
    return;
  }
  c[0] = id % D.d[0];
  c[1] = (id / D.d[0]) % D.d[1];
  c[2] = id / (D.d[0] * D.d[1]);
}

__device__ __forceinline__ int64_t vertex_of(const GradDims& D, const int64_t c[3]) {
  return (c[0] >> 1) + D.v[0] * ((c[1] >> 1) + D.v[1] * (c[2] >> 1));
}

// IsGreater on vertex indices (gi_regular_grid_trilinear_function.h:309-314)
__device__ __forceinline__ bool vert_greater(const float* f, int64_t a, int64_t b) {
  const float fa = f[a], fb = f[b];
  if (fa > fb) return true;
  if (fb > fa) return false;
  return a > b;
}

// Cell2HighestVertex of the hex at cell coords c (all axes odd)
__device__ __forceinline__ int64_t hex_highest(const float* f, const GradDims& D, const int64_t c[3]) {
  int64_t best = -1;
#pragma unroll
  for (int s = 0; s < 8; s++) {
    const int64_t v = ((c[0] >> 1) + (s & 1)) + D.v[0] * (((c[1] >> 1) + ((s >> 1) & 1)) + D.v[1] * ((c[2] >> 1) + (s >> 2)));
    if (best < 0 || vert_greater(f, v, best)) best = v;
  }
  return best;
}

// ComputeMINBoundary, pass `dim`: edges whose vertices carry different ascending labels
// (neither -1) get 1; then quads with a facet edge at 1; then hexes with a facet quad at 1.
__global__ void restrict_min_kernel(const int32_t* __restrict__ asc, const GradDims D, int dim,
                                    uint8_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D.ncells; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t c[3];
    cell_xyz(D, i, c);
    const int odd = (int)(c[0] & 1) + (int)(c[1] & 1) + (int)(c[2] & 1);
    if (odd != dim) continue;
    if (dim == 1) {
      const int a = (c[0] & 1) ? 0 : ((c[1] & 1) ? 1 : 2);
      int64_t lo[3] = {c[0], c[1], c[2]}, hi[3] = {c[0], c[1], c[2]};
      lo[a] -= 1;
      hi[a] += 1;
      const int32_t l1 = asc[vertex_of(D, lo)], l2 = asc[vertex_of(D, hi)];
      if (l1 != -1 && l2 != -1 && l1 != l2) out[i] = 1;
    } else {
      bool any = false;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        if (!(c[a] & 1)) continue;
        any |= out[i + D.cs[a]] == 1 || out[i - D.cs[a]] == 1;
      }
      if (any) out[i] = 1;
    }
  }
}

// ComputeMAXBoundary, pass `dim` (interior cells only): quads whose two hexes' highest
// vertices differ and carry different descending labels get +2; then edges with a
// cofacet quad above 1; then vertices with a cofacet edge above 1.
__global__ void restrict_max_kernel(const int32_t* __restrict__ dsc, const float* __restrict__ f, const GradDims D,
                                    int dim, uint8_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D.ncells; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t c[3];
    cell_xyz(D, i, c);
    const int odd = (int)(c[0] & 1) + (int)(c[1] & 1) + (int)(c[2] & 1);
    if (odd != dim) continue;
    bool interior = true;
#pragma unroll
    for (int a = 0; a < 3; a++) interior &= c[a] != 0 && c[a] != D.d[a] - 1;
    if (!interior) continue;
    if (dim == 2) {
      const int a = !(c[0] & 1) ? 0 : (!(c[1] & 1) ? 1 : 2);
      int64_t h1[3] = {c[0], c[1], c[2]}, h2[3] = {c[0], c[1], c[2]};
      h1[a] += 1;
      h2[a] -= 1;
      const int64_t v1 = hex_highest(f, D, h1), v2 = hex_highest(f, D, h2);
      if (v1 == v2) continue;  // the same lower star
      const int32_t l1 = dsc[v1], l2 = dsc[v2];
      if (l1 == -1 || l2 == -1 || l1 == l2) continue;
      out[i] = (uint8_t)(out[i] + 2);
    } else {
      bool any = false;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        if (c[a] & 1) continue;
        any |= out[i + D.cs[a]] > 1 || out[i - D.cs[a]] > 1;
      }
      if (any) out[i] = (uint8_t)(out[i] + 2);
    }
  }
}

// The re-pairing: one thread per vertex (lstar_core.cuh::conform_vertex).  The few
// touched vertices recompute their lower star; the rest only read 27 restriction bytes.
__global__ void __launch_bounds__(128) conform_kernel(const float* __restrict__ f, const uint8_t* __restrict__ rlab,
                                                      uint8_t* __restrict__ g, const GradDims D,
                                                      unsigned long long* __restrict__ touched) {
  using N = Nb<3>;
  const int64_t X = D.v[0], Y = D.v[1], Z = D.v[2];
  const int64_t nv = X * Y * Z;
  uint64_t col[27];
  unsigned long long n = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = v % X, y = (v / X) % Y, z = v / (X * Y);
    const float* fv = f + v;
    const int64_t c0 = 2 * x + 2 * y * D.cs[1] + 2 * z * D.cs[2];
    auto cell = [&](int p) { return c0 + N::d(p, 0) + N::d(p, 1) * D.cs[1] + N::d(p, 2) * D.cs[2]; };
    auto load = [&](int p, float& val) { val = __ldg(fv + (N::d(p, 0) + N::d(p, 1) * X + N::d(p, 2) * X * Y)); };
    auto rl = [&](int p, uint8_t& r) { r = rlab[cell(p)]; };
    auto store = [&](int p, uint8_t b) { g[cell(p)] = b; };
    const bool interior = x > 0 && x < X - 1 && y > 0 && y < Y - 1 && z > 0 && z < Z - 1;
    n += conform_vertex<3>(x, y, z, X, Y, Z, interior, load, rl, col, 1, D.enc_map, store);
  }
  if (n) atomicAdd(touched, n);
}

// Every cell's ldir back to the closure roots (critical 1-, 2-, 3-cells 2, 1, 0; the
// rest 3), so that the ldir stage recomputes the closure of the new pairing.
__global__ void ldir_roots_kernel(uint8_t* __restrict__ g, const GradDims D) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D.ncells; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t c[3];
    cell_xyz(D, i, c);
    const int dim = (int)(c[0] & 1) + (int)(c[1] & 1) + (int)(c[2] & 1);
    const uint8_t b = g[i];
    const bool crit = ((b >> 2) & 7) == 7;
    const int ldir = crit ? (dim == 1 ? 2 : (dim == 2 ? 1 : (dim == 3 ? 0 : 3))) : 3;
    g[i] = (uint8_t)((b & 0x1F) | (ldir << 5));
  }
}

}  // namespace

cudaError_t launch_restriction_labels(const int32_t* asc, const int32_t* dsc, const float* f, const GradDims& D,
                                      uint8_t* out, int num_sms, cudaStream_t stream) {
  if (cudaError_t e = cudaMemsetAsync(out, 0, (size_t)D.ncells, stream)) return e;
  const int grid = num_sms * 16;
  if (asc)
    for (int dim = 1; dim <= 3; dim++) {
      ::msc::count_launch();
      restrict_min_kernel<<<grid, 256, 0, stream>>>(asc, D, dim, out);
    }
  if (dsc)
    for (int dim = 2; dim >= 0; dim--) {
      ::msc::count_launch();
      restrict_max_kernel<<<grid, 256, 0, stream>>>(dsc, f, D, dim, out);
    }
  return cudaGetLastError();
}

cudaError_t launch_conform(const float* f, const uint8_t* rlab, uint8_t* g, const GradDims& D,
                           unsigned long long* touched, int num_sms, cudaStream_t stream) {
  ::msc::count_launch();
  conform_kernel<<<num_sms * 16, 128, 0, stream>>>(f, rlab, g, D, touched);
  ::msc::count_launch();
  ldir_roots_kernel<<<num_sms * 16, 256, 0, stream>>>(g, D);
  return cudaGetLastError();
}

}  // namespace msc
