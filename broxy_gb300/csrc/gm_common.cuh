// gm_common.cuh — shared device helpers for the GB300 GMorpho kernels.
//
// Layout conventions (identical to the reference library, so device buffers
// cross the C ABI without conversion):
//   * packed grid: uint8[res^3]; byte c = cx + res*cy + res*res*cz holds the
//     2x2x2 fine voxels 2c + (i,j,k) at bit i + 2j + 4k
//     (GMorpho/Grid.h:57-64, GMorpho/Voxelizer.cu:815-823);
//   * fine fields (radius grid, distance fields): x-fastest, N = 2*res per
//     axis (GMorpho/ScaleField.cu:61-72).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define GM_HD __host__ __device__ __forceinline__

namespace gm {

// 16-bit saturating cap used by every distance field ("no site in reach").
constexpr uint16_t kCap16 = 0xffff;

GM_HD int clamp_radius(int s) { return s < 2 ? 2 : (s > 127 ? 127 : s); }

GM_HD int64_t cell_index(int x, int y, int z, int res) {
  return (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
}
GM_HD int64_t fine_index(int x, int y, int z, int n) {
  return (int64_t)x + (int64_t)n * y + (int64_t)n * n * z;
}
// x-fastest index in a box of nx * ny * (any) elements
GM_HD int64_t idx3(int x, int y, int z, int nx, int ny) {
  return (int64_t)x + (int64_t)nx * y + (int64_t)nx * ny * z;
}
GM_HD int child_bit(int x, int y, int z) { return (x & 1) | ((y & 1) << 1) | ((z & 1) << 2); }

// Morton code with 10 bits per axis, x in bit 0 (GMorpho/cuda_math.h:111-117,
// 148-152).  Written with the usual magic-number spread.
GM_HD uint32_t spread_bits3(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
GM_HD uint32_t gather_bits3(uint32_t v) {
  v &= 0x09249249u;
  v = (v | (v >> 2)) & 0x030c30c3u;
  v = (v | (v >> 4)) & 0x0300f00fu;
  v = (v | (v >> 8)) & 0x030000ffu;
  v = (v | (v >> 16)) & 0x3ffu;
  return v;
}
GM_HD uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  return spread_bits3(x) | (spread_bits3(y) << 1) | (spread_bits3(z) << 2);
}

// 1-D box distance from lattice point p to voxel q = p + delta, in voxels:
// the distance to the nearer endpoint of [q, q+1] (GMorpho/cuda_math.h:973-988
// evaluated per axis).
GM_HD int lattice_dist(int delta) { return delta >= 0 ? delta : -delta - 1; }
// 1-D box distance from the centre of voxel p to voxel p + delta, in half voxels.
GM_HD int center_dist2(int delta) {
  int a = delta < 0 ? -delta : delta;
  return a == 0 ? 0 : 2 * a - 1;
}

__device__ __forceinline__ uint16_t min_u16(uint32_t a, uint32_t b) { return (uint16_t)(a < b ? a : b); }

}  // namespace gm
