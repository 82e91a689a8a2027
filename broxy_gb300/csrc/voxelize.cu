// voxelize.cu — conservative solid voxelization into the packed grid
// (reference row a2: Voxelizer::VoxelizeConservative, VoxelizeVolume,
// VoxelizeSurfaceConservative, ConvertBucketToPacketGrid;
// GMorpho/Voxelizer.cu:594-849 and the shaders vol_vox_bit.frag:35-51,
// surf_vox_conserv.geo:41-122, surf_vox_conserv_bit.frag:35-47).
//
// The reference rasterises with OpenGL (parity fill at pixel centres plus
// NVIDIA conservative rasterisation).  Here both passes are CUDA kernels
// with a precise definition (double precision, no contraction):
//   (i)  volume: a triangle covers pixel (x, y) when the pixel centre is
//        inside its xy projection (top-left rule on edges); it flips every
//        voxel of that column at or below floor(z at the centre);
//   (ii) surface: every voxel whose closed box meets the triangle
//        (separating-axis test) is set; triangles with squared aspect ratio
//        >= 50^2 are skipped as the geometry shader does (Voxelizer.cu:680).
// Both passes work on z-word bit grids (32 consecutive z per uint32, the
// reference's GL bucket layout), which are then packed into 2x2x2 bytes.
#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

size_t voxelize_scratch_bytes(int res) {
  const size_t N = 2 * (size_t)res;
  return 2 * (N * N * N / 8) + 512;
}

__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ bool edge_covers(double ax, double ay, double bx, double by, double px, double py) {
  const double w = dsub(dmul(dsub(bx, ax), dsub(py, ay)), dmul(dsub(by, ay), dsub(px, ax)));
  if (w > 0) return true;
  if (w < 0) return false;
  const double ex = dsub(bx, ax), ey = dsub(by, ay);
  return (ey == 0 && ex < 0) || (ey < 0);
}

__device__ bool tri_box_overlap(const double c[3], double half, const double v0[3], const double v1[3],
                                const double v2[3]) {
  double a[3], b[3], d[3];
  for (int i = 0; i < 3; i++) {
    a[i] = dsub(v0[i], c[i]);
    b[i] = dsub(v1[i], c[i]);
    d[i] = dsub(v2[i], c[i]);
  }
  for (int ax = 0; ax < 3; ax++) {
    const double mn = fmin(a[ax], fmin(b[ax], d[ax])), mx = fmax(a[ax], fmax(b[ax], d[ax]));
    if (mn > half || mx < -half) return false;
  }
  double e[3][3];
  for (int i = 0; i < 3; i++) {
    e[0][i] = dsub(b[i], a[i]);
    e[1][i] = dsub(d[i], b[i]);
    e[2][i] = dsub(a[i], d[i]);
  }
  const double nrm[3] = {dsub(dmul(e[0][1], e[1][2]), dmul(e[0][2], e[1][1])),
                         dsub(dmul(e[0][2], e[1][0]), dmul(e[0][0], e[1][2])),
                         dsub(dmul(e[0][0], e[1][1]), dmul(e[0][1], e[1][0]))};
  const double dd = dadd(dadd(dmul(nrm[0], a[0]), dmul(nrm[1], a[1])), dmul(nrm[2], a[2]));
  const double rr = dmul(half, dadd(dadd(fabs(nrm[0]), fabs(nrm[1])), fabs(nrm[2])));
  if (dd > rr || dd < -rr) return false;
  const double* vv[3] = {a, b, d};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double ax[3] = {0, 0, 0};
      if (j == 0) { ax[1] = -e[i][2]; ax[2] = e[i][1]; }
      if (j == 1) { ax[0] = e[i][2]; ax[2] = -e[i][0]; }
      if (j == 2) { ax[0] = -e[i][1]; ax[1] = e[i][0]; }
      double p[3];
      for (int k = 0; k < 3; k++) p[k] = dadd(dadd(dmul(ax[0], vv[k][0]), dmul(ax[1], vv[k][1])), dmul(ax[2], vv[k][2]));
      const double mn = fmin(p[0], fmin(p[1], p[2])), mx = fmax(p[0], fmax(p[1], p[2]));
      const double r = dmul(half, dadd(dadd(fabs(ax[0]), fabs(ax[1])), fabs(ax[2])));
      if (mn > r || mx < -r) return false;
    }
  return true;
}

__device__ __forceinline__ void set_zbit(uint32_t* g, int N, int x, int y, int z, bool xor_mode) {
  uint32_t* w = g + ((int64_t)x + (int64_t)N * y) * (N >> 5) + (z >> 5);
  const uint32_t m = 1u << (z & 31);
  if (xor_mode) atomicXor(w, m);
  else atomicOr(w, m);
}

__global__ void k_voxelize_tris(const float* __restrict__ P, const uint32_t* __restrict__ T, int64_t nf, int N,
                                double bx, double by, double bz, double h, uint32_t* __restrict__ mark,
                                uint32_t* __restrict__ surf) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nf; t += (int64_t)gridDim.x * blockDim.x) {
    double g[3][3];
    const double bb[3] = {bx, by, bz};
    for (int j = 0; j < 3; j++)
      for (int a = 0; a < 3; a++)
        g[j][a] = __ddiv_rn(dsub((double)P[3 * (size_t)T[3 * t + j] + a], bb[a]), h);
    // (i) volume parity
    double area = dsub(dmul(dsub(g[1][0], g[0][0]), dsub(g[2][1], g[0][1])),
                       dmul(dsub(g[1][1], g[0][1]), dsub(g[2][0], g[0][0])));
    if (area != 0) {
      int o1 = 1, o2 = 2;
      if (area < 0) { o1 = 2; o2 = 1; area = -area; }
      const double* A = g[0];
      const double* B = g[o1];
      const double* Cc = g[o2];
      const double mnx = fmin(A[0], fmin(B[0], Cc[0])), mxx = fmax(A[0], fmax(B[0], Cc[0]));
      const double mny = fmin(A[1], fmin(B[1], Cc[1])), mxy = fmax(A[1], fmax(B[1], Cc[1]));
      int x0 = (int)floor(mnx - 0.5), x1 = (int)ceil(mxx - 0.5);
      int y0 = (int)floor(mny - 0.5), y1 = (int)ceil(mxy - 0.5);
      x0 = max(x0, 0); y0 = max(y0, 0);
      x1 = min(x1, N - 1); y1 = min(y1, N - 1);
      for (int y = y0; y <= y1; y++)
        for (int x = x0; x <= x1; x++) {
          const double px = x + 0.5, py = y + 0.5;
          if (!edge_covers(A[0], A[1], B[0], B[1], px, py)) continue;
          if (!edge_covers(B[0], B[1], Cc[0], Cc[1], px, py)) continue;
          if (!edge_covers(Cc[0], Cc[1], A[0], A[1], px, py)) continue;
          const double wa = dsub(dmul(dsub(B[0], px), dsub(Cc[1], py)), dmul(dsub(B[1], py), dsub(Cc[0], px)));
          const double wb = dsub(dmul(dsub(Cc[0], px), dsub(A[1], py)), dmul(dsub(Cc[1], py), dsub(A[0], px)));
          const double wc = dsub(dsub(area, wa), wb);
          const double z = __ddiv_rn(dadd(dadd(dmul(wa, A[2]), dmul(wb, B[2])), dmul(wc, Cc[2])), area);
          int k = (int)floor(z);
          if (k < 0) continue;
          if (k > N - 1) k = N - 1;
          set_zbit(mark, N, x, y, k, true);
        }
    }
    // (ii) conservative surface
    double d0[3], d1[3], d2[3];
    for (int a = 0; a < 3; a++) {
      d0[a] = dsub(g[0][a], g[1][a]);
      d1[a] = dsub(g[1][a], g[2][a]);
      d2[a] = dsub(g[2][a], g[0][a]);
    }
    const double l0 = dadd(dadd(dmul(d0[0], d0[0]), dmul(d0[1], d0[1])), dmul(d0[2], d0[2]));
    const double l1 = dadd(dadd(dmul(d1[0], d1[0]), dmul(d1[1], d1[1])), dmul(d1[2], d1[2]));
    const double l2 = dadd(dadd(dmul(d2[0], d2[0]), dmul(d2[1], d2[1])), dmul(d2[2], d2[2]));
    double maxl2 = l0 > l1 ? l0 : l1;
    if (l2 > maxl2) maxl2 = l2;
    const double cx = dsub(dmul(d0[1], d2[2]), dmul(d0[2], d2[1]));
    const double cy = dsub(dmul(d0[2], d2[0]), dmul(d0[0], d2[2]));
    const double cz = dsub(dmul(d0[0], d2[1]), dmul(d0[1], d2[0]));
    const double a2 = dadd(dadd(dmul(cx, cx), dmul(cy, cy)), dmul(cz, cz));
    if (!(a2 > 0) || !(__ddiv_rn(dmul(maxl2, maxl2), a2) < 2500.0)) continue;
    // voxels x whose closed box [x, x + 1] meets [mn, mx] on every axis:
    // ceil(mn) - 1 <= x <= floor(mx) (the box test of tri_box_overlap, so
    // the voxels outside could not pass it)
    int lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
      const double mn = fmin(g[0][a], fmin(g[1][a], g[2][a])), mx = fmax(g[0][a], fmax(g[1][a], g[2][a]));
      lo[a] = max((int)ceil(mn) - 1, 0);
      hi[a] = min((int)floor(mx), N - 1);
    }
    for (int z = lo[2]; z <= hi[2]; z++)
      for (int y = lo[1]; y <= hi[1]; y++)
        for (int x = lo[0]; x <= hi[0]; x++) {
          const double c[3] = {x + 0.5, y + 0.5, z + 0.5};
          if (tri_box_overlap(c, 0.5, g[0], g[1], g[2])) set_zbit(surf, N, x, y, z, false);
        }
  }
}

// parity: voxel z of a column is set when an odd number of marks sit at
// or above it; combined with the surface bits in place (into `mark`).
__global__ void k_parity_columns(uint32_t* __restrict__ mark, const uint32_t* __restrict__ surf, int N) {
  const int64_t cols = (int64_t)N * N;
  const int W = N >> 5;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < cols; c += (int64_t)gridDim.x * blockDim.x) {
    uint32_t* m = mark + c * W;
    const uint32_t* s = surf + c * W;
    uint32_t carry = 0;  // parity of all marks above this word
    for (int w = W - 1; w >= 0; w--) {
      uint32_t x = m[w];
      // suffix xor toward lower bits: bit i = xor of bits >= i
      x ^= x >> 1;
      x ^= x >> 2;
      x ^= x >> 4;
      x ^= x >> 8;
      x ^= x >> 16;
      x ^= carry ? 0xffffffffu : 0u;
      carry = x & 1u;
      m[w] = x | s[w];
    }
  }
}

__global__ void k_zwords_to_packed(const uint32_t* __restrict__ zw, uint8_t* __restrict__ grid, int res) {
  const int N = 2 * res, W = N >> 5;
  const int64_t total = (int64_t)res * res * res;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < total; c += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(c % res), y = (int)((c / res) % res), z = (int)(c / ((int64_t)res * res));
    uint8_t b = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
      const uint32_t w = zw[((int64_t)fx + (int64_t)N * fy) * W + (fz >> 5)];
      b |= (uint8_t)(((w >> (fz & 31)) & 1u) << k);
    }
    grid[c] = b;
  }
}

__global__ void k_packed_to_zwords(const uint8_t* __restrict__ grid, uint32_t* __restrict__ zw, int res) {
  const int N = 2 * res, W = N >> 5;
  const int64_t total = (int64_t)N * N * W;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int kz = (int)(i % W);
    const int64_t col = i / W;
    const int fx = (int)(col % N), fy = (int)(col / N);
    uint32_t w = 0;
    for (int j = 0; j < 32; j++) {
      const int fz = 32 * kz + j;
      const uint8_t b = grid[cell_index(fx >> 1, fy >> 1, fz >> 1, res)];
      w |= (uint32_t)((b >> child_bit(fx, fy, fz)) & 1u) << j;
    }
    zw[i] = w;
  }
}

static int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_voxelize(const float* P, int64_t nv, const uint32_t* T, int64_t nf, int res,
                            const float* bbox_min, float cell_size, uint8_t* grid, uint8_t* scratch,
                            cudaStream_t st, KernelCounter* kc) {
  (void)nv;
  const int N = 2 * res;
  const size_t words = (size_t)N * N * N / 32;
  uint32_t* mark = reinterpret_cast<uint32_t*>(scratch);
  uint32_t* surf = mark + words;
  cudaMemsetAsync(mark, 0, 2 * words * sizeof(uint32_t), st);
  const double h = 0.5 * (double)cell_size;
  if (nf > 0) {
    int b = (int)((nf + 127) / 128);
    if (b > 152 * 64) b = 152 * 64;
    GM_LAUNCH(kc, "k_voxelize_tris", st, k_voxelize_tris<<<b, 128, 0, st>>>(P, T, nf, N, (double)bbox_min[0], (double)bbox_min[1], (double)bbox_min[2],
                                       h, mark, surf));
  }
  GM_LAUNCH(kc, "k_parity_columns", st, k_parity_columns<<<blocks_for((int64_t)N * N), 256, 0, st>>>(mark, surf, N));
  GM_LAUNCH(kc, "k_zwords_to_packed", st, k_zwords_to_packed<<<blocks_for((int64_t)res * res * res), 256, 0, st>>>(mark, grid, res));
  return cudaGetLastError();
}

cudaError_t launch_layout(int res, const uint32_t* zw, uint8_t* grid, int dir, cudaStream_t st, KernelCounter* kc) {
  if (dir == 0) GM_LAUNCH(kc, "k_zwords_to_packed", st, k_zwords_to_packed<<<blocks_for((int64_t)res * res * res), 256, 0, st>>>(zw, grid, res));
  else {
    const int N = 2 * res;
    GM_LAUNCH(kc, "k_packed_to_zwords", st, k_packed_to_zwords<<<blocks_for((int64_t)N * N * (N / 32)), 256, 0, st>>>(grid, const_cast<uint32_t*>(zw), res));
  }
  return cudaGetLastError();
}

}  // namespace gm
