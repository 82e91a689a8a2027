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
// * Shortcuts from the squared lattice distance field E of the input grid
//   (launch_edt): the cube of half size r contains the ball of radius r and
//   lies in the ball of radius r sqrt(3), so E(p) < r^2 is a hit and
//   E(p) >= 3 (r + 1)^2 a miss.  Both keep a margin of at least 1/(2r)
//   fine voxels to the float predicate's decision, far above its rounding
//   (about 1e-4 at these coordinates), so they never change a boolean.
//   Only the shell between them is searched.
// * The search gives each such query one warp: the warp takes up to four
//   pending nodes of its current level and its 32 lanes test their 32
//   children at once (one child box per lane), the survivors are compacted
//   into the next level's list (at most 32 entries per level, so 12 x 32
//   entries bound the whole search), and the first surviving fine voxel
//   ends it.  A per-lane depth-first search left 3 to 8 of 32 lanes active
//   per instruction (neighbouring queries descend through different node
//   counts).
// * Base pass: cells inside data_res whose byte is not 0xff; frame at the
//   cell, centre 2c, radius of fine voxel 2c.  Contour: the cells whose byte
//   differs from a diagonal neighbour (ComputeContourBaseConservative,
//   GMorpho/Grid.cu:1464-1498, 2170-2230), listed with warp-aggregated
//   atomics; their eight fine voxels (frame on the 2 res lattice, own
//   radius) overwrite the byte.
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

// The occupancy pyramid: level 0 is the input grid (a node's bits are its
// fine voxels), levels 1..L ((res >> l)^3 node bytes) follow each other in
// `up`, level l at byte (8^L - 8^(L-l+1)) / 7.
struct RcLevels {
  const uint8_t* X;
  const uint8_t* up;
  int L;  // log2(res)
  __host__ __device__ __forceinline__ const uint8_t* level(int l) const {
    return l == 0 ? X : up + ((((int64_t)1 << (3 * L)) - ((int64_t)1 << (3 * (L - l + 1)))) / 7);
  }
  const uint8_t* level_host(int l) const { return level(l); }
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
// axes of the rotated cube and the box (centre n, half size hs).  All 15
// comparisons are evaluated (no early exit) so that the lanes of a warp,
// each testing another box, stay together; the boolean is the same.
__device__ __forceinline__ bool rc_overlap(const RcQuery& q, float nx, float ny, float nz, float hs) {
  const float tx = q.c[0] - nx, ty = q.c[1] - ny, tz = q.c[2] - nz;
  const float* bx = q.bx;
  const float* by = q.by;
  const float* bz = q.bz;
  const float se = q.se;
  bool sep = fabsf(tx) > hs + se * (fabsf(bx[0]) + fabsf(by[0]) + fabsf(bz[0]));
  sep |= fabsf(ty) > hs + se * (fabsf(bx[1]) + fabsf(by[1]) + fabsf(bz[1]));
  sep |= fabsf(tz) > hs + se * (fabsf(bx[2]) + fabsf(by[2]) + fabsf(bz[2]));
  sep |= fabsf(tx * bx[0] + ty * bx[1] + tz * bx[2]) > hs * (fabsf(bx[0]) + fabsf(bx[1]) + fabsf(bx[2])) + se;
  sep |= fabsf(tx * by[0] + ty * by[1] + tz * by[2]) > hs * (fabsf(by[0]) + fabsf(by[1]) + fabsf(by[2])) + se;
  sep |= fabsf(tx * bz[0] + ty * bz[1] + tz * bz[2]) > hs * (fabsf(bz[0]) + fabsf(bz[1]) + fabsf(bz[2])) + se;
  sep |= fabsf(tz * bx[1] - ty * bx[2]) > hs * (fabsf(bx[2]) + fabsf(bx[1])) + se * (fabsf(bz[0]) + fabsf(by[0]));
  sep |= fabsf(tz * by[1] - ty * by[2]) > hs * (fabsf(by[2]) + fabsf(by[1])) + se * (fabsf(bz[0]) + fabsf(bx[0]));
  sep |= fabsf(tz * bz[1] - ty * bz[2]) > hs * (fabsf(bz[2]) + fabsf(bz[1])) + se * (fabsf(by[0]) + fabsf(bx[0]));
  sep |= fabsf(tx * bx[2] - tz * bx[0]) > hs * (fabsf(bx[2]) + fabsf(bx[0])) + se * (fabsf(bz[1]) + fabsf(by[1]));
  sep |= fabsf(tx * by[2] - tz * by[0]) > hs * (fabsf(by[2]) + fabsf(by[0])) + se * (fabsf(bz[1]) + fabsf(bx[1]));
  sep |= fabsf(tx * bz[2] - tz * bz[0]) > hs * (fabsf(bz[2]) + fabsf(bz[0])) + se * (fabsf(by[1]) + fabsf(bx[1]));
  sep |= fabsf(ty * bx[0] - tx * bx[1]) > hs * (fabsf(bx[1]) + fabsf(bx[0])) + se * (fabsf(bz[2]) + fabsf(by[2]));
  sep |= fabsf(ty * by[0] - tx * by[1]) > hs * (fabsf(by[1]) + fabsf(by[0])) + se * (fabsf(bz[2]) + fabsf(bx[2]));
  sep |= fabsf(ty * bz[0] - tx * bz[1]) > hs * (fabsf(bz[1]) + fabsf(bz[0])) + se * (fabsf(by[2]) + fabsf(bx[2]));
  return !sep;
}

__device__ __forceinline__ int rc_radius(const int8_t* __restrict__ R, int uniform_r, int fx, int fy, int fz, int n) {
  return clamp_radius(R ? (int)__ldg(R + fine_index(fx, fy, fz, n)) : uniform_r);
}

// Decision from the squared lattice distance e (saturated, a lower bound of
// the true one) of the query point to the nearest occupied fine voxel box:
// 1 = dilated, 0 = not dilated, -1 = search.
// * e < r^2: a voxel box reaches into the ball of radius r, which the cube
//   of half size r contains with a margin of at least 1/(2r) fine voxels
//   along every axis (also for each box containing that voxel box, i.e. the
//   voxel's pyramid ancestors), against float rounding of about 1e-4 here.
// * A voxel box passing the predicate passes its separating-axis tests 1-3
//   (box within se * A_i of the query along axis i, A_i = |b_x,i| + |b_y,i|
//   + |b_z,i|) and 4-6 (its centre within se + w_j / 2 of the query along
//   b_j, w_j = |b_j,x| + |b_j,y| + |b_j,z|), so it lies at squared distance
//   at most M1 = sum_i (se A_i)^2 and at most M2 = (sum_j (se + w_j / 2)^2
//   ^ 1/2 + 0.01)^2 (0.01 covers the tests' float rounding).  e > min(M1, M2)
//   leaves no voxel that could pass: not dilated, exactly.
__device__ __forceinline__ int rc_shortcut(const RcQuery& q, uint32_t e) {
  const float r = q.se;
  if ((float)e < r * r) return 1;
  const float* b[3] = {q.bx, q.by, q.bz};
  float m1 = 0.f, m2 = 0.f;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float h = q.se * (fabsf(q.bx[i]) + fabsf(q.by[i]) + fabsf(q.bz[i]));
    m1 += h * h;
    const float g = q.se + 0.5f * (fabsf(b[i][0]) + fabsf(b[i][1]) + fabsf(b[i][2]));
    m2 += g * g;
  }
  m2 = sqrtf(m2) + 0.01f;
  m2 *= m2;
  // float rounding of these bounds: a few ulps, covered by 1e-5 relative
  const float m = (m1 < m2 ? m1 : m2) * 1.00001f + 1e-3f;
  if ((float)e > m) return 0;  // NaN axes: m is NaN, no decision
  return -1;
}

__device__ __forceinline__ uint64_t rc_pack(int x, int y, int z) {
  return (uint64_t)x | ((uint64_t)y << 21) | ((uint64_t)z << 42);
}

constexpr int kRcSearchWarps = kRcThreads / 32;

// One warp, one query.  Each round the warp takes up to NPL pending nodes
// of its level; lane l tests 8 / (32 / NPL) children of node l / (32 / NPL)
// (the lanes of a node start with the children away from the query, so that
// the compacted list ends with the nearest ones, which are taken first);
// the surviving children become the next level's pending list and the warp
// descends.  A level's list only receives children while it is empty (the
// warp climbs back only once a level is exhausted), so it never holds more
// than 8 NPL nodes.  True at the first surviving fine voxel.  Warp-uniform
// control flow; the per-level counts (<= 64) live in three registers.
template <int NPL>
__device__ bool rc_search(const RcLevels& P, const RcQuery& q, uint64_t (*lst)[8 * NPL], int lane) {
  constexpr int LPN = 32 / NPL;  // lanes per node
  constexpr int CPL = 8 / LPN;   // children per lane
  const int maxd = P.L + 1;
  uint32_t c0 = 1, c1 = 0, c2 = 0;  // 8-bit pending counts of levels 0..11
  auto getc = [&](int d) -> int {
    const uint32_t w = d < 4 ? c0 : (d < 8 ? c1 : c2);
    return (int)((w >> ((d & 3) * 8)) & 0xffu);
  };
  auto setc = [&](int d, int v) {
    const int sh = (d & 3) * 8;
    const uint32_t m = ~(0xffu << sh), x = (uint32_t)v << sh;
    if (d < 4) c0 = (c0 & m) | x;
    else if (d < 8) c1 = (c1 & m) | x;
    else c2 = (c2 & m) | x;
  };
  if (lane == 0) lst[0][0] = rc_pack(0, 0, 0);
  int d = 0;
  // each round consumes at least one pending node; the pending nodes are
  // finite (a tree), so the loop ends
  for (;;) {
    __syncwarp();
    const int cd = getc(d);
    if (cd == 0) {
      if (d == 0) return false;
      d--;
      continue;
    }
    const int m = cd < NPL ? cd : NPL;
    setc(d, cd - m);
    const int j = lane / LPN;
    bool ok[CPL];
    uint64_t child[CPL];
#pragma unroll
    for (int u = 0; u < CPL; u++) ok[u] = false, child[u] = 0;
    if (j < m) {
      const uint64_t nd = lst[d][cd - m + j];
      const int nx = (int)(nd & 0x1fffff), ny = (int)((nd >> 21) & 0x1fffff), nz = (int)(nd >> 42);
      const int level = P.L - d;
      const int64_t nl = (int64_t)1 << d;
      const uint32_t occ = __ldg(P.level(level) + nx + nl * ny + nl * nl * nz);
      const float ns = (float)(2 << level);
      const int near = (q.c[0] >= ns * ((float)nx + 0.5f)) | ((q.c[1] >= ns * ((float)ny + 0.5f)) << 1) |
                       ((q.c[2] >= ns * ((float)nz + 0.5f)) << 2);
      const float ncs = (float)(1 << level);  // child size: 2 res >> (d + 1)
#pragma unroll
      for (int u = 0; u < CPL; u++) {
        const int t = (lane % LPN) * CPL + u;  // 7 = the child on the query's side
        const int k = t ^ near ^ 7;
        if ((occ >> k) & 1) {
          const int cx = 2 * nx + (k & 1), cy = 2 * ny + ((k >> 1) & 1), cz = 2 * nz + (k >> 2);
          ok[u] = rc_overlap(q, ncs * ((float)cx + 0.5f), ncs * ((float)cy + 0.5f), ncs * ((float)cz + 0.5f),
                             0.5f * ncs);
          child[u] = rc_pack(cx, cy, cz);
        }
      }
    }
    uint32_t surv[CPL];
    int tot = 0;
#pragma unroll
    for (int u = 0; u < CPL; u++) {
      surv[u] = __ballot_sync(0xffffffffu, ok[u]);
      tot += __popc(surv[u]);
    }
    if (tot == 0) continue;
    if (d + 1 == maxd) return true;
    __syncwarp();
    int at = 0;
#pragma unroll
    for (int u = 0; u < CPL; u++) {
      if (ok[u]) lst[d + 1][at + __popc(surv[u] & ((1u << lane) - 1))] = child[u];
      at += __popc(surv[u]);
    }
    setc(d + 1, tot);
    d++;
  }
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

// warp-aggregated append of (cell, voxel mask) entries
__device__ __forceinline__ void rc_append(bool want, uint64_t entry, uint64_t* __restrict__ list,
                                          uint32_t* __restrict__ count, int lane) {
  const uint32_t bal = __ballot_sync(0xffffffffu, want);
  if (bal == 0) return;
  uint32_t at = 0;
  if (lane == 0) at = atomicAdd(count, (uint32_t)__popc(bal));
  at = __shfl_sync(0xffffffffu, at, 0);
  if (want) list[at + __popc(bal & ((1u << lane) - 1))] = entry;
}

// DilateByRotCubeByTexMipmapBase, decided part: D[c] = X[c], or 0xff when
// the corner 2c is dilated by the distance shortcut; the undecided cells are
// listed for rc_search
__global__ void __launch_bounds__(kRcThreads) k_rc_base_cls(const uint8_t* __restrict__ X,
                                                            const uint16_t* __restrict__ E,
                                                            const int8_t* __restrict__ R, int uniform_r,
                                                            const float4* __restrict__ Q, int qres, int res, int dx,
                                                            int dy, int dz, uint8_t* __restrict__ D,
                                                            uint64_t* __restrict__ list, uint32_t* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  const int64_t total = (int64_t)res * res * res, stride = (int64_t)gridDim.x * blockDim.x;
  const int N = 2 * res;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
    const int64_t c = base + lane;
    bool search = false;
    if (c < total) {
      const int x = (int)(c % res), y = (int)((c / res) % res), z = (int)(c / ((int64_t)res * res));
      const uint8_t v = X[c];
      uint8_t out = v;
      if (v != 0xff && x < dx && y < dy && z < dz) {
        RcQuery q;
        rc_frame(Q, qres, x, y, z, res, q);
        q.c[0] = (float)(2 * x), q.c[1] = (float)(2 * y), q.c[2] = (float)(2 * z);
        q.se = (float)rc_radius(R, uniform_r, 2 * x, 2 * y, 2 * z, N);
        const int s = E ? rc_shortcut(q, __ldg(E + fine_index(2 * x, 2 * y, 2 * z, N))) : -1;
        if (s == 1) out = 0xff;
        search = s < 0;
      }
      D[c] = out;
    }
    rc_append(search, ((uint64_t)c << 8) | 1u, list, count, lane);
  }
}

// TagVoxelsContourBaseConservative on D, appended to tags
__global__ void __launch_bounds__(kRcThreads) k_rc_tag(const uint8_t* __restrict__ D, int res,
                                                       uint32_t* __restrict__ tags, uint32_t* __restrict__ count) {
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
    if (tag) tags[at + __popc(bal & ((1u << lane) - 1))] = (uint32_t)c;
  }
}

// DilateByRotCubeByTexMipmap, decided part: one thread per cell (tags, or
// every cell when tags is null: GM_EXACT) writes the byte of its fine voxels
// decided by the distance shortcut and lists the others for rc_search
__global__ void __launch_bounds__(kRcThreads) k_rc_fine_cls(const uint16_t* __restrict__ E,
                                                            const int8_t* __restrict__ R, int uniform_r,
                                                            const float4* __restrict__ Q, int qres, int res,
                                                            const uint32_t* __restrict__ tags,
                                                            const uint32_t* __restrict__ ntags,
                                                            uint8_t* __restrict__ D, uint64_t* __restrict__ list,
                                                            uint32_t* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  const int64_t total = tags ? (int64_t)*ntags : (int64_t)res * res * res;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int N = 2 * res;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
    const int64_t i = base + lane;
    uint32_t undecided = 0;
    int64_t c = 0;
    if (i < total) {
      c = tags ? (int64_t)tags[i] : i;
      const int x = (int)(c % res), y = (int)((c / res) % res), z = (int)(c / ((int64_t)res * res));
      uint32_t hit = 0;
      for (int k = 0; k < 8; k++) {
        const int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
        RcQuery q;
        rc_frame(Q, qres, fx, fy, fz, N, q);
        q.c[0] = (float)fx, q.c[1] = (float)fy, q.c[2] = (float)fz;
        q.se = (float)rc_radius(R, uniform_r, fx, fy, fz, N);
        const int s = E ? rc_shortcut(q, __ldg(E + fine_index(fx, fy, fz, N))) : -1;
        if (s == 1) hit |= 1u << k;
        if (s < 0) undecided |= 1u << k;
      }
      D[c] = (uint8_t)hit;
    }
    rc_append(undecided != 0, ((uint64_t)c << 8) | undecided, list, count, lane);
  }
}

// The listed queries, one warp each (rc_search).  Base entries (fine == 0):
// corner 2c of the cell, frame on the res lattice, D[c] = 0xff on a hit.
// Fine entries: the voxels of the mask, frame on the 2 res lattice, hit
// bits or-ed into D[c] (one entry per cell: no other writer).
template <int NPL>
__global__ void __launch_bounds__(kRcThreads, 2) k_rc_search(RcLevels P, const int8_t* __restrict__ R, int uniform_r,
                                                          const float4* __restrict__ Q, int qres, int res,
                                                          const uint64_t* __restrict__ list,
                                                          const uint32_t* __restrict__ count,
                                                          uint32_t* __restrict__ next, int fine,
                                                          uint8_t* __restrict__ D) {
  __shared__ uint64_t lst[kRcSearchWarps][kRotCubeMaxLevels][8 * NPL];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n = *count;
  const int N = 2 * res;
  // entries are taken one at a time from a shared counter: their costs
  // differ by orders of magnitude, a fixed split would leave warps idle
  for (;;) {
    uint32_t e = 0;
    if (lane == 0) e = atomicAdd(next, 1u);
    e = __shfl_sync(0xffffffffu, e, 0);
    if ((int64_t)e >= n) break;
    const uint64_t ent = list[e];
    const int64_t c = (int64_t)(ent >> 8);
    uint32_t mask = (uint32_t)(ent & 0xff);
    const int x = (int)(c % res), y = (int)((c / res) % res), z = (int)(c / ((int64_t)res * res));
    uint32_t hits = 0;
    while (mask) {
      const int k = __ffs(mask) - 1;
      mask &= mask - 1;
      RcQuery q;
      if (fine) {
        const int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
        rc_frame(Q, qres, fx, fy, fz, N, q);
        q.c[0] = (float)fx, q.c[1] = (float)fy, q.c[2] = (float)fz;
        q.se = (float)rc_radius(R, uniform_r, fx, fy, fz, N);
      } else {
        rc_frame(Q, qres, x, y, z, res, q);
        q.c[0] = (float)(2 * x), q.c[1] = (float)(2 * y), q.c[2] = (float)(2 * z);
        q.se = (float)rc_radius(R, uniform_r, 2 * x, 2 * y, 2 * z, N);
      }
      if (rc_search<NPL>(P, q, lst[w], lane)) hits |= 1u << k;
    }
    if (lane == 0 && hits) D[c] = fine ? (uint8_t)(D[c] | hits) : (uint8_t)0xff;
  }
}

int ilog2_exact(int v) {
  int l = 0;
  while ((1 << l) < v) l++;
  return (1 << l) == v ? l : -1;
}

}  // namespace

// occupancy levels 1..L (contiguous), the tag list (u32 per cell) and the
// search list (u64 per cell), with their counters
size_t rotcube_scratch_bytes(int res) {
  const size_t cells = (size_t)res * res * res;
  const size_t up = (cells - 1) / 7;  // sum of (res >> l)^3, l = 1..L
  return ((up + 255) & ~(size_t)255) + 256 + ((4 * cells + 255) & ~(size_t)255) + 8 * cells;
}

template <int NPL>
static void launch_search(const RcLevels& P, const RotCubeArgs& a, const float4* Q, const uint64_t* list,
                          const uint32_t* count, uint32_t* next, int fine, int blocks, cudaStream_t st,
                          KernelCounter* kc) {
  cudaMemsetAsync(next, 0, sizeof(uint32_t), st);
  GM_LAUNCH(kc, "k_rc_search", st,
            k_rc_search<NPL><<<blocks, kRcThreads, 0, st>>>(P, a.R, a.uniform_r, Q, a.qres, a.res, list, count, next,
                                                            fine, a.D));
}

cudaError_t launch_rotcube_dilation(const RotCubeArgs& a, cudaStream_t st, KernelCounter* kc) {
  const int res = a.res;
  const int L = ilog2_exact(res);
  if (L < 1 || L + 1 > kRotCubeMaxLevels || a.qres < 1 || !a.X || !a.Q || !a.D || !a.scratch)
    return cudaErrorInvalidValue;
  const size_t cells = (size_t)res * res * res;
  RcLevels P{};
  P.L = L;
  P.X = a.X;
  P.up = a.scratch;
  uint8_t* p = a.scratch + (((cells - 1) / 7 + 255) & ~(size_t)255);
  uint32_t* counts = reinterpret_cast<uint32_t*>(p);  // [0] tags, [1] search list, [2] next entry
  p += 256;
  uint32_t* tags = reinterpret_cast<uint32_t*>(p);
  p += (4 * cells + 255) & ~(size_t)255;
  uint64_t* list = reinterpret_cast<uint64_t*>(p);
  // the distance field of the shortcuts first (launch_edt uses the
  // scratch region as its own temporaries): saturated at (re + 1)^2, with
  // re >= every radius (hits are decided below r^2) and, up to 127, beyond
  // the largest miss bound
  if (a.E) {
    // the largest miss bound M2 is (sqrt(3) (rmax + sqrt(3) / 2) + 0.01)^2
    int re = (int)(1.7321f * (float)a.rmax) + 3;
    if (re > 127) re = 127;
    if (re < a.rmax) return cudaErrorInvalidValue;
    cudaError_t e = launch_edt(a.X, res, re, a.edt_workspace, a.E, st, kc);
    if (e != cudaSuccess) return e;
  }
  for (int l = 1; l <= L; l++) {
    const int nf = res >> (l - 1);
    const int64_t nt = (int64_t)(nf / 2) * (nf / 2) * (nf / 2);
    int b = (int)((nt + 255) / 256);
    if (b > 152 * 16) b = 152 * 16;
    GM_LAUNCH(kc, "k_rc_occ_up", st,
              k_rc_occ_up<<<b, 256, 0, st>>>(P.level_host(l - 1), nf, const_cast<uint8_t*>(P.level_host(l))));
  }
  const float4* Q = reinterpret_cast<const float4*>(a.Q);
  const int sms = a.num_sms > 0 ? a.num_sms : 152;
  const int grid = sms * 8;
  // four nodes per round measured faster than one, two or eight (the
  // searched queries expand many nodes: breadth pays, up to the 32 lanes)
  auto search = [&](int fine) { launch_search<4>(P, a, Q, list, counts + 1, counts + 2, fine, sms * 2, st, kc); };
  cudaMemsetAsync(counts, 0, 2 * sizeof(uint32_t), st);
  if (a.mode == 0) {
    GM_LAUNCH(kc, "k_rc_base_cls", st,
              k_rc_base_cls<<<grid, kRcThreads, 0, st>>>(a.X, a.E, a.R, a.uniform_r, Q, a.qres, res, a.data_res[0],
                                                         a.data_res[1], a.data_res[2], a.D, list, counts + 1));
    search(0);
    GM_LAUNCH(kc, "k_rc_tag", st, k_rc_tag<<<grid, kRcThreads, 0, st>>>(a.D, res, tags, counts));
    cudaMemsetAsync(counts + 1, 0, sizeof(uint32_t), st);
    GM_LAUNCH(kc, "k_rc_fine_cls", st,
              k_rc_fine_cls<<<grid, kRcThreads, 0, st>>>(a.E, a.R, a.uniform_r, Q, a.qres, res, tags, counts, a.D,
                                                         list, counts + 1));
  } else {
    GM_LAUNCH(kc, "k_rc_fine_cls", st,
              k_rc_fine_cls<<<grid, kRcThreads, 0, st>>>(a.E, a.R, a.uniform_r, Q, a.qres, res, nullptr, counts,
                                                         a.D, list, counts + 1));
  }
  search(1);
  return cudaGetLastError();
}

}  // namespace gm
