// scalefield.cu — ScaleField brush update (reference row a3:
// ScaleField::UpdateGrid / UpdateScaleGrid / tukey,
// GMorpho/ScaleField.cu:81-141, 148-202; GMorpho/cuda_math.h:696-704).
//
// The float operations are written with explicit rounding (no contraction
// other than the two fused multiply-adds spelled out below) so that the
// result is bit-identical to the host restatement.
#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

// One warp per fine row (y, z) of the brush box, lanes along x (coalesced
// bytes).  A row is skipped when its squared distance with ux = 0 already
// fails the test: rounding is monotone and every term is non-negative, so
// fma(uz, uz, fma(uy, uy, ux*ux)) >= fma(uz, uz, fma(uy, uy, 0)) for every
// x, and the per-voxel test below could not pass either.
__global__ void __launch_bounds__(256) k_scale_brush(int8_t* __restrict__ R, int n, float bx, float by, float bz,
                                                     float cell, float px, float py, float pz, float v, float h,
                                                     float target, int mode, int x0, int y0, int z0, int x1, int y1,
                                                     int z1) {
  const int wx = x1 - x0 + 1, wy = y1 - y0 + 1, wz = z1 - z0 + 1;
  const int lane = threadIdx.x & 31;
  const int64_t rows = (int64_t)wy * wz;
  const float reach = __fadd_rn(v, h);
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < rows;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int y = y0 + (int)(r % wy), z = z0 + (int)(r / wy);
    const float uy = __fsub_rn(__fmaf_rn(cell, (float)y, by), py);
    const float uz = __fsub_rn(__fmaf_rn(cell, (float)z, bz), pz);
    if (!(__fsqrt_rn(__fmaf_rn(uz, uz, __fmaf_rn(uy, uy, 0.f))) < reach)) continue;  // warp-uniform
    const int64_t row = fine_index(0, y, z, n);
    for (int x = x0 + lane; x < x0 + wx; x += 32) {
      const float ux = __fsub_rn(__fmaf_rn(cell, (float)x, bx), px);
      const float d = __fsqrt_rn(__fmaf_rn(uz, uz, __fmaf_rn(uy, uy, __fmul_rn(ux, ux))));
      if (!(d < reach)) continue;
      float w;
      if (d < v) {
        w = 1.f;
      } else {
        const float a = __fdiv_rn(__fsub_rn(d, v), h);
        const float b = __fsub_rn(1.f, __fmul_rn(a, a));
        w = __fmul_rn(b, b);
      }
      const int64_t idx = row + x;
      const float prev = (float)R[idx];
      float dist = __fadd_rn(__fmul_rn(prev, __fsub_rn(1.f, w)), __fmul_rn(w, target));
      dist = floorf(dist);
      dist = fmaxf(fminf(dist, 127.f), 0.f);
      if (mode == 1) R[idx] = (int8_t)floorf(fmaxf(dist, prev));
      else if (mode == 2) R[idx] = (int8_t)floorf(fminf(dist, prev));
      else if (mode == 3) R[idx] = (int8_t)dist;
    }
  }
}

cudaError_t launch_scale_brush(int8_t* R, int n, const float* bbox_min, float cell_size, const float* pos,
                               float scale, float support, float global_scale, int mode, cudaStream_t st,
                               KernelCounter* kc) {
  const float v = scale;
  const float h = (support - v) / sqrtf(1.f - sqrtf(0.5f));
  const float target = mode == 3 ? global_scale / cell_size : scale / cell_size;
  // Only voxels with d < v + h change; bound them by a box (the reference
  // sweeps the whole grid, GMorpho/ScaleField.cu:171-182).
  const float reach = v + h;
  int lo[3], hi[3];
  for (int a = 0; a < 3; a++) {
    const float l = (pos[a] - reach - bbox_min[a]) / cell_size;
    const float u = (pos[a] + reach - bbox_min[a]) / cell_size;
    lo[a] = (int)floorf(l) - 1;
    hi[a] = (int)ceilf(u) + 1;
    if (!(reach == reach) || !(l == l)) { lo[a] = 0; hi[a] = n - 1; }
    if (lo[a] < 0) lo[a] = 0;
    if (hi[a] > n - 1) hi[a] = n - 1;
  }
  if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) return cudaSuccess;
  const int64_t rows = (int64_t)(hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
  int64_t blocks = (rows + 7) / 8;  // a warp per row
  if (blocks > 152 * 32) blocks = 152 * 32;
  GM_LAUNCH(kc, "k_scale_brush", st, k_scale_brush<<<(unsigned)blocks, 256, 0, st>>>(R, n, bbox_min[0], bbox_min[1], bbox_min[2], cell_size, pos[0], pos[1],
                                        pos[2], v, h, target, mode, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]));
  return cudaGetLastError();
}

}  // namespace gm
