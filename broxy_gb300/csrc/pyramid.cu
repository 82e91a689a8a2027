// pyramid.cu — the OR / max-radius texel pyramid (reference row a4:
// Grid::BuildTexMipmaps(const ScaleField&), FillLevel0, BuildMipmapFromTo;
// GMorpho/Grid.cu:957-1154, 733-805).
//
// Texel layout kept identical to the reference so that the pyramid can be
// exchanged through the C ABI: bits 56..63 = child k occupied, bits
// 7k..7k+6 = radius of child k (level 0: the clamped fine radius; above: the
// maximum over the child's eight radius fields, occupied or not).  Levels are
// stored linearly (x-fastest) and concatenated from level 0 to the root.
// The closing itself does not traverse this pyramid (it uses separable
// transforms), so the build is offered as a standalone operator.
#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

size_t pyramid_texels(int res) {
  size_t t = 0;
  for (int n = res; n >= 1; n >>= 1) t += (size_t)n * n * n;
  return t;
}

__global__ void k_pyr_level0(const uint8_t* __restrict__ grid, const int8_t* __restrict__ R, int uniform_r, int res,
                             uint64_t* __restrict__ out) {
  const int N = 2 * res;
  const int64_t total = (int64_t)res * res * res;
  const int ru = clamp_radius(uniform_r);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < total; c += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(c % res), y = (int)((c / res) % res), z = (int)(c / ((int64_t)res * res));
    uint64_t t = grid[c];
#pragma unroll
    for (int k = 7; k >= 0; k--) {
      const int r = R ? clamp_radius(R[fine_index(2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2), N)])
                      : ru;
      t = (t << 7) | (uint64_t)(r & 0x7f);
    }
    out[c] = t;
  }
}

__global__ void k_pyr_up(const uint64_t* __restrict__ from, int nf, uint64_t* __restrict__ to) {
  const int nt = nf >> 1;
  const int64_t total = (int64_t)nt * nt * nt;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nt), y = (int)((i / nt) % nt), z = (int)(i / ((int64_t)nt * nt));
    uint64_t out = 0, occ = 0;
#pragma unroll
    for (int k = 7; k >= 0; k--) {
      const uint64_t v = from[cell_index(2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2), nf)];
      uint32_t m = 0;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const uint32_t r = (uint32_t)(v >> (7 * j)) & 0x7fu;
        m = r > m ? r : m;
      }
      out = (out << 7) | m;
      occ |= (uint64_t)((v >> 56) != 0) << k;
    }
    to[i] = out | (occ << 56);
  }
}

cudaError_t launch_pyramid(const uint8_t* grid, const int8_t* R, int uniform_r, int res, uint64_t* pyr,
                           cudaStream_t st, KernelCounter* kc) {
  const int64_t n0 = (int64_t)res * res * res;
  int blocks = (int)((n0 + 255) / 256);
  if (blocks > 152 * 32) blocks = 152 * 32;
  GM_LAUNCH(kc, "k_pyr_level0", st, k_pyr_level0<<<blocks, 256, 0, st>>>(grid, R, uniform_r, res, pyr));
  uint64_t* from = pyr;
  for (int n = res; n > 1; n >>= 1) {
    uint64_t* to = from + (size_t)n * n * n;
    const int64_t nt = (int64_t)(n / 2) * (n / 2) * (n / 2);
    int b = (int)((nt + 255) / 256);
    if (b > 152 * 32) b = 152 * 32;
    GM_LAUNCH(kc, "k_pyr_up", st, k_pyr_up<<<b, 256, 0, st>>>(from, n, to));
    from = to;
  }
  return cudaGetLastError();
}

}  // namespace gm
