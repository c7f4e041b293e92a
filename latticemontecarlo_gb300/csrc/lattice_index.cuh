// Site ids and half-unit coordinates of the FCC supercells (device side), shared by
// the kernels of kernels.cu and the fused surrogate kernel (mlp_fused.cu).
// Ids follow Config::ReassignLatticeVector (lmc/cfg/src/Config.cpp:466-552):
// id = hx * 2 n^2 + hy * n + hz / 2 for half-unit coordinates (hx, hy, hz) in [0, 2n).
#pragma once

#include <cuda_runtime.h>

namespace lmc {

struct H3 {
  int x, y, z;
};

__device__ __forceinline__ H3 SiteCoord(long long id, int n) {
  // 32-bit unsigned arithmetic: supercells have n <= 1000, so 4 n^3 < 2^32
  const unsigned u = static_cast<unsigned>(id), nn = static_cast<unsigned>(n);
  const unsigned plane = 2u * nn * nn;
  const unsigned hx = u / plane;
  const unsigned r = u - hx * plane;
  const unsigned hy = r / nn;
  const unsigned k = r - hy * nn;
  return {static_cast<int>(hx), static_cast<int>(hy), static_cast<int>(2 * k + ((hx + hy) & 1u))};
}

// Id of h + (dx, dy, dz) with periodic wrap; |offset| <= 4 < 2n. 32-bit unsigned
// arithmetic: (x 2n + y) n + z / 2 < 4 n^3 < 2^32 for n <= 1000.
__device__ __forceinline__ long long NeighborId(H3 h, int dx, int dy, int dz, int n) {
  const int m = 2 * n;
  int x = h.x + dx, y = h.y + dy, z = h.z + dz;
  x += (x < 0) ? m : 0;
  x -= (x >= m) ? m : 0;
  y += (y < 0) ? m : 0;
  y -= (y >= m) ? m : 0;
  z += (z < 0) ? m : 0;
  z -= (z >= m) ? m : 0;
  const unsigned nn = static_cast<unsigned>(n);
  return static_cast<long long>((static_cast<unsigned>(x) * 2u * nn + static_cast<unsigned>(y)) * nn +
                                (static_cast<unsigned>(z) >> 1));
}

// h + (dx, dy, dz) with periodic wrap (half units); |offset| <= 4 < 2n.
__device__ __forceinline__ H3 WrapCoord(H3 h, int dx, int dy, int dz, int n) {
  const int m = 2 * n;
  int x = h.x + dx, y = h.y + dy, z = h.z + dz;
  x += (x < 0) ? m : 0;
  x -= (x >= m) ? m : 0;
  y += (y < 0) ? m : 0;
  y -= (y >= m) ? m : 0;
  z += (z < 0) ? m : 0;
  z -= (z >= m) ? m : 0;
  return {x, y, z};
}

__device__ __forceinline__ int MinImage(int d, int n) {
  const int m = 2 * n;
  d %= m;
  if (d < -n) d += m;
  if (d >= n) d -= m;
  return d;
}

// Minimum image of a coordinate difference d in (-2n, 2n) (half units).
__device__ __forceinline__ int WrapDelta(int d, int n) {
  d += d < -n ? 2 * n : 0;
  d -= d >= n ? 2 * n : 0;
  return d;
}

}  // namespace lmc
