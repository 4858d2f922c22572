// Host build of the CUDA lower-star core (msceer_gb300/csrc/lstar_core.cuh) for the
// CPU tests: the very code the kernel runs per vertex, driven over a whole volume,
// so its parity with the oracle is checked without a GPU.
#include <cstdint>

#include "../msceer_gb300/csrc/lstar_core.cuh"

template <int ND>
static int run(const float* f, int64_t X, int64_t Y, int64_t Z, uint8_t* g, uint32_t enc_map) {
  using N = msc::Nb<ND>;
  const int64_t dX = 2 * X - 1, dY = 2 * Y - 1;
  const int64_t cs1 = dX, cs2 = dX * dY;
  uint64_t col[27];
  int nan = 0;
  for (int64_t z = 0; z < Z; z++)
    for (int64_t y = 0; y < Y; y++)
      for (int64_t x = 0; x < X; x++) {
        const float* fv = f + x + X * (y + Y * z);
        uint8_t* gc = g + 2 * x + 2 * y * cs1 + 2 * z * cs2;
        auto load = [&](int p, float& v) {
          v = fv[N::d(p, 0) + N::d(p, 1) * X + (ND == 3 ? N::d(p, 2) : 0) * X * Y];
        };
        auto store = [&](int p, uint8_t b) {
          gc[N::d(p, 0) + N::d(p, 1) * cs1 + (ND == 3 ? N::d(p, 2) : 0) * cs2] = b;
        };
        const bool interior = x > 0 && x < X - 1 && y > 0 && y < Y - 1 && (ND == 2 || (z > 0 && z < Z - 1));
        nan |= msc::process_vertex<ND>(x, y, z, X, Y, Z, interior, load, col, 1, enc_map, store);
      }
  return nan;
}

extern "C" int core_pairs_3d(const float* f, int64_t X, int64_t Y, int64_t Z, uint8_t* g, uint32_t enc_map) {
  return run<3>(f, X, Y, Z, g, enc_map);
}
extern "C" int core_pairs_2d(const float* f, int64_t X, int64_t Y, uint8_t* g, uint32_t enc_map) {
  return run<2>(f, X, Y, 1, g, enc_map);
}

// The conforming re-pairing of every vertex (restriction labels per cell), pairs and
// ldir roots of the recomputed lower stars written into g.
extern "C" int core_conform_3d(const float* f, int64_t X, int64_t Y, int64_t Z, const uint8_t* rlab, uint8_t* g,
                               uint32_t enc_map) {
  using N = msc::Nb<3>;
  const int64_t dX = 2 * X - 1, dY = 2 * Y - 1;
  const int64_t cs1 = dX, cs2 = dX * dY;
  uint64_t col[27];
  int n = 0;
  for (int64_t z = 0; z < Z; z++)
    for (int64_t y = 0; y < Y; y++)
      for (int64_t x = 0; x < X; x++) {
        const float* fv = f + x + X * (y + Y * z);
        const int64_t c0 = 2 * x + 2 * y * cs1 + 2 * z * cs2;
        auto load = [&](int p, float& v) { v = fv[N::d(p, 0) + N::d(p, 1) * X + N::d(p, 2) * X * Y]; };
        auto cell = [&](int p) { return c0 + N::d(p, 0) + N::d(p, 1) * cs1 + N::d(p, 2) * cs2; };
        auto rl = [&](int p, uint8_t& r) { r = rlab[cell(p)]; };
        auto store = [&](int p, uint8_t b) { g[cell(p)] = b; };
        const bool interior = x > 0 && x < X - 1 && y > 0 && y < Y - 1 && z > 0 && z < Z - 1;
        n += msc::conform_vertex<3>(x, y, z, X, Y, Z, interior, load, rl, col, 1, enc_map, store);
      }
  return n;
}
