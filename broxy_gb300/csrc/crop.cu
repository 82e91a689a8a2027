// crop.cu — byte-box copies between cubic grids and the occupied extent of
// a packed grid: the crops of the edit server (crop, write-back) and of the
// batched closings (closing on the occupied extent, embedding back).
#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

// Copy of the box [s, s + e) of a cubic byte volume of edge sn into the box
// [d, d + e) of a cubic volume of edge dn; one block per row.  Callers keep
// both boxes inside their volumes.
__global__ void k_box_copy(const uint8_t* __restrict__ src, int sn, int sx, int sy, int sz, uint8_t* __restrict__ dst,
                           int dn, int dx, int dy, int dz, int ex) {
  const int y = blockIdx.x, z = blockIdx.y;
  const uint8_t* s = src + cell_index(sx, sy + y, sz + z, sn);
  uint8_t* d = dst + cell_index(dx, dy + y, dz + z, dn);
  for (int x = threadIdx.x; x < ex; x += blockDim.x) d[x] = s[x];
}

cudaError_t launch_box_copy(const uint8_t* src, int sn, const int s0[3], uint8_t* dst, int dn, const int d0[3],
                            const int ext[3], cudaStream_t st, KernelCounter* kc) {
  if (ext[0] <= 0 || ext[1] <= 0 || ext[2] <= 0) return cudaSuccess;
  const int threads = ext[0] >= 256 ? 256 : 128;
  GM_LAUNCH(kc, "k_box_copy", st,
            k_box_copy<<<dim3(ext[1], ext[2]), threads, 0, st>>>(src, sn, s0[0], s0[1], s0[2], dst, dn, d0[0], d0[1],
                                                                 d0[2], ext[0]));
  return cudaGetLastError();
}

// Whole grid C (edge res) from the crop Cc (edge ext, at the origin): the
// crop's bytes inside it, zeros elsewhere.  One block per row of C.
__global__ void k_embed(const uint8_t* __restrict__ Cc, int ext, uint8_t* __restrict__ C, int res) {
  const int y = blockIdx.x, z = blockIdx.y;
  uint8_t* d = C + cell_index(0, y, z, res);
  const bool row_in = y < ext && z < ext;
  const uint8_t* s = Cc + cell_index(0, row_in ? y : 0, row_in ? z : 0, ext);
  for (int x = threadIdx.x; x < res; x += blockDim.x) d[x] = (row_in && x < ext) ? s[x] : (uint8_t)0;
}

cudaError_t launch_embed(const uint8_t* Cc, int ext, uint8_t* C, int res, cudaStream_t st, KernelCounter* kc) {
  GM_LAUNCH(kc, "k_embed", st, k_embed<<<dim3(res, res), res >= 256 ? 256 : 128, 0, st>>>(Cc, ext, C, res));
  return cudaGetLastError();
}

// 1 + the largest x, y and z of a non-empty cell (0 for an empty grid),
// accumulated into out[0..2] (which the caller zeroes).  res^3 is a
// multiple of 16: one 16-byte word per step.
__global__ void k_occ_extent(const uint8_t* __restrict__ X, int res, int64_t words, unsigned* __restrict__ out) {
  unsigned mx = 0, my = 0, mz = 0;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < words; w += (int64_t)gridDim.x * blockDim.x) {
    const uint4 v = reinterpret_cast<const uint4*>(X)[w];
    if ((v.x | v.y | v.z | v.w) == 0u) continue;
    const uint32_t q[4] = {v.x, v.y, v.z, v.w};
    int last = -1;
#pragma unroll
    for (int k = 0; k < 16; k++)
      if ((q[k >> 2] >> (8 * (k & 3))) & 0xffu) last = k;
    int first = 16;
#pragma unroll
    for (int k = 15; k >= 0; k--)
      if ((q[k >> 2] >> (8 * (k & 3))) & 0xffu) first = k;
    const int64_t c0 = 16 * w + first, c1 = 16 * w + last;
    // a word holds 16 consecutive cells of one row when res >= 16
    const unsigned y = (unsigned)((c0 / res) % res), z = (unsigned)(c0 / ((int64_t)res * res));
    mx = max(mx, (unsigned)(c1 % res) + 1u);
    my = max(my, y + 1u);
    mz = max(mz, z + 1u);
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  my = __reduce_max_sync(0xffffffffu, my);
  mz = __reduce_max_sync(0xffffffffu, mz);
  if ((threadIdx.x & 31) == 0 && (mx | my | mz) != 0u) {
    atomicMax(out + 0, mx);
    atomicMax(out + 1, my);
    atomicMax(out + 2, mz);
  }
}

cudaError_t launch_occ_extent(const uint8_t* X, int res, unsigned* d_out3, int sms, cudaStream_t st,
                              KernelCounter* kc) {
  cudaMemsetAsync(d_out3, 0, 3 * sizeof(unsigned), st);
  const int64_t words = (int64_t)res * res * res / 16;
  int64_t blocks = (words + 255) / 256;
  const int64_t cap = (int64_t)(sms > 0 ? sms : 152) * 8;
  if (blocks > cap) blocks = cap;
  GM_LAUNCH(kc, "k_occ_extent", st, k_occ_extent<<<(int)blocks, 256, 0, st>>>(X, res, words, d_out3));
  return cudaGetLastError();
}

}  // namespace gm
