// rotcube.cu — rotated-cube dilation under a frame field (reference:
// GMorpho::DilateByRotCubeMipmap, GMorpho/GMorpho.cu:3058-3230, with the
// kernels DilateByRotCubeByTexMipmapBase, GMorpho.cu:1712-1837, and
// DilateByRotCubeByTexMipmap, GMorpho.cu:2464-2602).
//
// The structuring element at a lattice point p is the cube of half size
// r(p) centred on p and rotated by the frame field's quaternion
// interpolated at p.  It is not separable, so this dilation keeps the
// reference's hierarchical search: an occupancy byte pyramid over the input
// grid (bit k of a node = child k holds any voxel) is descended while the
// children's boxes overlap the rotated cube (separating-axis test), and the
// point is dilated as soon as one occupied fine voxel is reached.
//
// * The descent keeps one 8-bit "children still to visit" mask per level
//   (at most 12 levels) instead of the reference's 64-entry node stack, and
//   stops at the first reached voxel (the reference keeps popping; the
//   boolean is the same).
// * Base pass: one thread per cell inside data_res whose byte is not 0xff,
//   frame at the cell, centre 2c, radius of fine voxel 2c.
// * Contour: the cells whose byte differs from a diagonal neighbour
//   (ComputeContourBaseConservative, GMorpho/Grid.cu:1464-1498, 2170-2230)
//   are appended to a list with warp-aggregated atomics; then eight lanes
//   per listed cell (one per fine voxel, frame on the 2 res grid) search
//   and one ballot assembles the cell's byte.
//
// Every float expression is the reference's, evaluated left to right; this
// translation unit is compiled with -fmad=false so that no multiply-add is
// fused, and division and square root are IEEE round-to-nearest, as in the
// CPU oracle (compiled with -ffp-contract=off): both give the same booleans.
#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

namespace {

constexpr int kRcThreads = 256;

struct RcLevels {
  const uint8_t* lv[kRotCubeMaxLevels];  // lv[0] = input grid, lv[l] = (res >> l)^3 node bytes
  int L;                                 // log2(res)
};

// the structuring element of one lattice point
struct RcQuery {
  float c[3];             // centre, fine units
  float bx[3], by[3], bz[3];
  float se;               // half size
};

__device__ __forceinline__ float4 rc_node(const float4* __restrict__ Q, int64_t n, int64_t i) {
  // past the last node: clamped (the reference reads beyond its field there)
  return __ldg(Q + (i < n ? i : n - 1));
}

__device__ __forceinline__ float4 rc_lerp(float4 a, float4 b, float t) {
  const float s = 1.f - t;
  return make_float4(s * a.x + t * b.x, s * a.y + t * b.y, s * a.z + t * b.z, s * a.w + t * b.w);
}

// Hamilton product, terms in the reference's order (cuda_math.h:386-393)
__device__ __forceinline__ float4 rc_mul(float4 a, float4 b) {
  float4 r;
  r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
  r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
  r.y = a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x;
  r.z = a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w;
  return r;
}

// InterpolateQuaternionField (GMorpho.cu:1631-1710: trilinear, group size
// 0 = plain weighted sums), normalize (conj (quat)) and the rotated axes
// rotate (quat, e_k) (GMorpho.cu:1735-1745; cuda_math.h:396-401)
__device__ void rc_frame(const float4* __restrict__ Q, int qres, int ix, int iy, int iz, int res, RcQuery& q) {
  const float fres = (float)res, fq = (float)qres;
  const float fx = fq * ((float)ix / fres), fy = fq * ((float)iy / fres), fz = fq * ((float)iz / fres);
  const int jx = (int)fx, jy = (int)fy, jz = (int)fz;
  const int64_t sy = qres, sz = (int64_t)qres * qres, n = sz * qres;
  const int64_t b = jx + sy * jy + sz * jz;
  const float tx = fx - (float)jx, ty = fy - (float)jy, tz = fz - (float)jz;
  const float4 q00 = rc_lerp(rc_node(Q, n, b), rc_node(Q, n, b + 1), tx);
  const float4 q01 = rc_lerp(rc_node(Q, n, b + sz), rc_node(Q, n, b + 1 + sz), tx);
  const float4 q10 = rc_lerp(rc_node(Q, n, b + sy), rc_node(Q, n, b + 1 + sy), tx);
  const float4 q11 = rc_lerp(rc_node(Q, n, b + sy + sz), rc_node(Q, n, b + 1 + sy + sz), tx);
  float4 u = rc_lerp(rc_lerp(q00, q10, ty), rc_lerp(q01, q11, ty), tz);
  u.x = -u.x;
  u.y = -u.y;
  u.z = -u.z;
  const float len = sqrtf(u.x * u.x + u.y * u.y + u.z * u.z + u.w * u.w);
  u.x = u.x / len;
  u.y = u.y / len;
  u.z = u.z / len;
  u.w = u.w / len;
  const float4 uc = make_float4(-u.x, -u.y, -u.z, u.w);
  float4 r = rc_mul(uc, rc_mul(make_float4(1.f, 0.f, 0.f, 0.f), u));
  q.bx[0] = r.x, q.bx[1] = r.y, q.bx[2] = r.z;
  r = rc_mul(uc, rc_mul(make_float4(0.f, 1.f, 0.f, 0.f), u));
  q.by[0] = r.x, q.by[1] = r.y, q.by[2] = r.z;
  r = rc_mul(uc, rc_mul(make_float4(0.f, 0.f, 1.f, 0.f), u));
  q.bz[0] = r.x, q.bz[1] = r.y, q.bz[2] = r.z;
}

// HasRotCubeSEOverlap (GMorpho.cu:241-302, 334-349): the 15 separating
// axes of the rotated cube and the node box (centre n, half size hs)
__device__ __forceinline__ bool rc_overlap(const RcQuery& q, float nx, float ny, float nz, float hs) {
  const float tx = q.c[0] - nx, ty = q.c[1] - ny, tz = q.c[2] - nz;
  const float* bx = q.bx;
  const float* by = q.by;
  const float* bz = q.bz;
  const float se = q.se;
  if (fabsf(tx) > hs + se * (fabsf(bx[0]) + fabsf(by[0]) + fabsf(bz[0]))) return false;
  if (fabsf(ty) > hs + se * (fabsf(bx[1]) + fabsf(by[1]) + fabsf(bz[1]))) return false;
  if (fabsf(tz) > hs + se * (fabsf(bx[2]) + fabsf(by[2]) + fabsf(bz[2]))) return false;
  if (fabsf(tx * bx[0] + ty * bx[1] + tz * bx[2]) > hs * (fabsf(bx[0]) + fabsf(bx[1]) + fabsf(bx[2])) + se) return false;
  if (fabsf(tx * by[0] + ty * by[1] + tz * by[2]) > hs * (fabsf(by[0]) + fabsf(by[1]) + fabsf(by[2])) + se) return false;
  if (fabsf(tx * bz[0] + ty * bz[1] + tz * bz[2]) > hs * (fabsf(bz[0]) + fabsf(bz[1]) + fabsf(bz[2])) + se) return false;
  if (fabsf(tz * bx[1] - ty * bx[2]) > hs * (fabsf(bx[2]) + fabsf(bx[1])) + se * (fabsf(bz[0]) + fabsf(by[0]))) return false;
  if (fabsf(tz * by[1] - ty * by[2]) > hs * (fabsf(by[2]) + fabsf(by[1])) + se * (fabsf(bz[0]) + fabsf(bx[0]))) return false;
  if (fabsf(tz * bz[1] - ty * bz[2]) > hs * (fabsf(bz[2]) + fabsf(bz[1])) + se * (fabsf(by[0]) + fabsf(bx[0]))) return false;
  if (fabsf(tx * bx[2] - tz * bx[0]) > hs * (fabsf(bx[2]) + fabsf(bx[0])) + se * (fabsf(bz[1]) + fabsf(by[1]))) return false;
  if (fabsf(tx * by[2] - tz * by[0]) > hs * (fabsf(by[2]) + fabsf(by[0])) + se * (fabsf(bz[1]) + fabsf(bx[1]))) return false;
  if (fabsf(tx * bz[2] - tz * bz[0]) > hs * (fabsf(bz[2]) + fabsf(bz[0])) + se * (fabsf(by[1]) + fabsf(bx[1]))) return false;
  if (fabsf(ty * bx[0] - tx * bx[1]) > hs * (fabsf(bx[1]) + fabsf(bx[0])) + se * (fabsf(bz[2]) + fabsf(by[2]))) return false;
  if (fabsf(ty * by[0] - tx * by[1]) > hs * (fabsf(by[1]) + fabsf(by[0])) + se * (fabsf(bz[2]) + fabsf(bx[2]))) return false;
  if (fabsf(ty * bz[0] - tx * bz[1]) > hs * (fabsf(bz[1]) + fabsf(bz[0])) + se * (fabsf(by[2]) + fabsf(bx[2]))) return false;
  return true;
}

// children of node (nx, ny, nz) at depth d that hold a voxel and overlap
__device__ __forceinline__ uint32_t rc_children(const RcLevels& P, const RcQuery& q, int d, int nx, int ny, int nz) {
  const int level = P.L - d;
  const int64_t nl = (int64_t)1 << d;
  const uint32_t occ = __ldg(P.lv[level] + nx + nl * ny + nl * nl * nz);
  if (occ == 0) return 0;
  const float ncs = (float)(1 << level);  // child size: 2 res >> (d + 1)
  const float hs = 0.5f * ncs;
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (!((occ >> k) & 1)) continue;
    const float cx = ncs * ((float)(2 * nx + (k & 1)) + 0.5f);
    const float cy = ncs * ((float)(2 * ny + ((k >> 1) & 1)) + 0.5f);
    const float cz = ncs * ((float)(2 * nz + (k >> 2)) + 0.5f);
    if (rc_overlap(q, cx, cy, cz, hs)) m |= 1u << k;
  }
  return m;
}

// depth-first descent; true at the first reached fine voxel
__device__ bool rc_find(const RcLevels& P, const RcQuery& q) {
  const int maxd = P.L + 1;
  uint32_t mask[kRotCubeMaxLevels];
  int d = 0, nx = 0, ny = 0, nz = 0;
  mask[0] = rc_children(P, q, 0, 0, 0, 0);
  // at most 8 children per node and maxd levels: the loop ends
  for (;;) {
    const uint32_t m = mask[d];
    if (m == 0) {
      if (d == 0) return false;
      d--;
      nx >>= 1, ny >>= 1, nz >>= 1;
      continue;
    }
    const int k = __ffs(m) - 1;
    mask[d] = m & (m - 1);
    if (d + 1 == maxd) return true;
    nx = 2 * nx + (k & 1), ny = 2 * ny + ((k >> 1) & 1), nz = 2 * nz + (k >> 2);
    d++;
    mask[d] = rc_children(P, q, d, nx, ny, nz);
  }
}

__device__ __forceinline__ int rc_radius(const int8_t* __restrict__ R, int uniform_r, int fx, int fy, int fz, int n) {
  return clamp_radius(R ? (int)__ldg(R + fine_index(fx, fy, fz, n)) : uniform_r);
}

// one node byte per thread: bit k = child k of the finer level non-empty
__global__ void k_rc_occ_up(const uint8_t* __restrict__ from, int nf, uint8_t* __restrict__ to) {
  const int nt = nf >> 1;
  const int64_t total = (int64_t)nt * nt * nt;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nt), y = (int)((i / nt) % nt), z = (int)(i / ((int64_t)nt * nt));
    uint32_t b = 0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      b |= (uint32_t)(from[cell_index(2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2), nf)] != 0) << k;
    to[i] = (uint8_t)b;
  }
}

// DilateByRotCubeByTexMipmapBase: D[c] = 0xff when the cell's corner 2c is
// dilated, else X[c]; cells outside data_res and full cells copy X
__global__ void __launch_bounds__(kRcThreads) k_rc_base(RcLevels P, const int8_t* __restrict__ R, int uniform_r,
                                                        const float4* __restrict__ Q, int qres, int res, int dx,
                                                        int dy, int dz, uint8_t* __restrict__ D) {
  const uint8_t* X = P.lv[0];
  const int64_t total = (int64_t)res * res * res;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < total; c += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(c % res), y = (int)((c / res) % res), z = (int)(c / ((int64_t)res * res));
    const uint8_t v = X[c];
    uint8_t out = v;
    if (v != 0xff && x < dx && y < dy && z < dz) {
      RcQuery q;
      rc_frame(Q, qres, x, y, z, res, q);
      q.c[0] = (float)(2 * x), q.c[1] = (float)(2 * y), q.c[2] = (float)(2 * z);
      q.se = (float)rc_radius(R, uniform_r, 2 * x, 2 * y, 2 * z, 2 * res);
      if (rc_find(P, q)) out = 0xff;
    }
    D[c] = out;
  }
}

// TagVoxelsContourBaseConservative on D, appended to list (order free:
// each listed cell is rewritten from the input grid alone)
__global__ void __launch_bounds__(kRcThreads) k_rc_tag(const uint8_t* __restrict__ D, int res,
                                                       uint32_t* __restrict__ list, uint32_t* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  const int64_t total = (int64_t)res * res * res;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t s1 = res, s2 = (int64_t)res * res;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
    const int64_t c = base + lane;
    bool tag = false;
    if (c < total) {
      const int x = (int)(c % res), y = (int)((c / res) % res), z = (int)(c / s2);
      if (x >= 1 && y >= 1 && z >= 1 && x <= res - 2 && y <= res - 2 && z <= res - 2) {
        const uint8_t v = D[c];
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const int64_t o = ((k & 1) ? 1 : -1) + s1 * (((k >> 1) & 1) ? 1 : -1) + s2 * ((k >> 2) ? 1 : -1);
          tag |= D[c + o] != v;
        }
      }
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, tag);
    if (bal == 0) continue;
    uint32_t at = 0;
    if (lane == 0) at = atomicAdd(count, (uint32_t)__popc(bal));
    at = __shfl_sync(0xffffffffu, at, 0);
    if (tag) list[at + __popc(bal & ((1u << lane) - 1))] = (uint32_t)c;
  }
}

// DilateByRotCubeByTexMipmap: eight lanes per cell (fine voxel k = lane & 7,
// frame on the 2 res grid, its own radius); one ballot makes the byte.
// Cells: list[0 .. *count) or, when list is null, every cell (GM_EXACT).
__global__ void __launch_bounds__(kRcThreads) k_rc_fine(RcLevels P, const int8_t* __restrict__ R, int uniform_r,
                                                        const float4* __restrict__ Q, int qres, int res,
                                                        const uint32_t* __restrict__ list,
                                                        const uint32_t* __restrict__ count, uint8_t* __restrict__ D) {
  const int lane = threadIdx.x & 31;
  const int64_t ncell = list ? (int64_t)*count : (int64_t)res * res * res;
  const int64_t total = 8 * ncell;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int N = 2 * res;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
    const int64_t i = base + lane;
    bool hit = false;
    int64_t c = 0;
    if (i < total) {
      c = list ? (int64_t)list[i >> 3] : (i >> 3);
      const int k = (int)(i & 7);
      const int x = (int)(c % res), y = (int)((c / res) % res), z = (int)(c / ((int64_t)res * res));
      const int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
      RcQuery q;
      rc_frame(Q, qres, fx, fy, fz, N, q);
      q.c[0] = (float)fx, q.c[1] = (float)fy, q.c[2] = (float)fz;
      q.se = (float)rc_radius(R, uniform_r, fx, fy, fz, N);
      hit = rc_find(P, q);
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, hit);
    if (i < total && (lane & 7) == 0) D[c] = (uint8_t)((bal >> lane) & 0xffu);
  }
}

int ilog2_exact(int v) {
  int l = 0;
  while ((1 << l) < v) l++;
  return (1 << l) == v ? l : -1;
}

}  // namespace

size_t rotcube_scratch_bytes(int res) {
  size_t t = 0;
  for (int n = res >> 1; n >= 1; n >>= 1) t += ((size_t)n * n * n + 255) & ~(size_t)255;
  return t + (size_t)4 * res * res * res + 512;
}

cudaError_t launch_rotcube_dilation(const RotCubeArgs& a, cudaStream_t st, KernelCounter* kc) {
  const int res = a.res;
  const int L = ilog2_exact(res);
  if (L < 1 || L + 1 > kRotCubeMaxLevels || a.qres < 1 || !a.X || !a.Q || !a.D || !a.scratch)
    return cudaErrorInvalidValue;
  RcLevels P{};
  P.L = L;
  P.lv[0] = a.X;
  uint8_t* p = a.scratch;
  for (int l = 1; l <= L; l++) {
    const int n = res >> l;
    P.lv[l] = p;
    p += ((size_t)n * n * n + 255) & ~(size_t)255;
  }
  uint32_t* count = reinterpret_cast<uint32_t*>(p);
  uint32_t* list = count + 64;
  // occupancy levels, finest first
  for (int l = 1; l <= L; l++) {
    const int nf = res >> (l - 1);
    const int64_t nt = (int64_t)(nf / 2) * (nf / 2) * (nf / 2);
    int b = (int)((nt + 255) / 256);
    if (b > 152 * 16) b = 152 * 16;
    GM_LAUNCH(kc, "k_rc_occ_up", st,
              k_rc_occ_up<<<b, 256, 0, st>>>(P.lv[l - 1], nf, const_cast<uint8_t*>(P.lv[l])));
  }
  const float4* Q = reinterpret_cast<const float4*>(a.Q);
  const int grid = a.num_sms > 0 ? a.num_sms * 8 : 152 * 8;
  if (a.mode == 0) {
    GM_LAUNCH(kc, "k_rc_base", st,
              k_rc_base<<<grid, kRcThreads, 0, st>>>(P, a.R, a.uniform_r, Q, a.qres, res, a.data_res[0],
                                                     a.data_res[1], a.data_res[2], a.D));
    cudaMemsetAsync(count, 0, sizeof(uint32_t), st);
    GM_LAUNCH(kc, "k_rc_tag", st, k_rc_tag<<<grid, kRcThreads, 0, st>>>(a.D, res, list, count));
    GM_LAUNCH(kc, "k_rc_fine", st,
              k_rc_fine<<<grid, kRcThreads, 0, st>>>(P, a.R, a.uniform_r, Q, a.qres, res, list, count, a.D));
  } else {
    GM_LAUNCH(kc, "k_rc_fine", st,
              k_rc_fine<<<grid, kRcThreads, 0, st>>>(P, a.R, a.uniform_r, Q, a.qres, res, nullptr, count, a.D));
  }
  return cudaGetLastError();
}

}  // namespace gm
