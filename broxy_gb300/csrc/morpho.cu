// morpho.cu — variable-radius ball/cube closing on GB300 (reference rows
// a5..a11: GMorpho::DilateBySphereMipmap / DilateByCubeMipmap /
// ErodeBySphereMipmap, GMorpho/GMorpho.cu:3231-3314, 3538-3596, 6627-6702).
//
// The reference answers every dilation/erosion predicate by a per-thread
// stack traversal of a texture pyramid.  Here the same predicates are
// computed as separable min-plus distance transforms over fine-voxel
// fields, one axis per pass, each pass a tiled, coalesced, HBM-streaming
// kernel:
//
//   dilation (query radius r(p), GMorpho.cu:2858-2867):
//       D(p) = min_q sum_a d_a(q - p)^2 < (r(p) + 1)^2   (sphere)
//       D(p) = max_a-combined L-inf lattice distance <= r(p)   (cube)
//     with d(delta) the distance from lattice point p to the box of voxel q.
//   erosion (source radius r(q), GMorpho.cu:4403-4411, 5283-5349):
//       E(s) = min_q [K - 4 (r(q)-1)^2 + sum_a e_a^2] < K,  q in contour S,
//     in half-voxel units (e = box distance from point s to voxel q),
//     K = 4 (rmax - 1)^2, at voxel centres (fine pass) and at the lattice
//     points 2c+1 (base pass).
//
// The two-level structure of the reference (base pass on whole cells,
// refinement of contour cells only) is then applied exactly by the select
// kernels, which reproduces the reference grids bit for bit (GM_REF), or
// skipped (GM_EXACT).
#include <cudaTypedefs.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "gm_common.cuh"
#include "gm_internal.h"
#include "tma.cuh"

namespace gm {

// Error bits recorded by kernels (kErrTmaTimeout, ...); read and cleared by
// kernel_error_flags().
__device__ unsigned int g_kernel_errors = 0;

// A radius field read in place: element (x, y, z) at p[x + y sy + z sz]
// (a whole field, or a crop of a larger one without copying it).
struct RField {
  const int8_t* p;
  int64_t sy, sz;
};
__device__ __forceinline__ int rget(const RField& f, int x, int y, int z) {
  return f.p[(int64_t)x + (int64_t)y * f.sy + (int64_t)z * f.sz];
}

// A box of cells [lo, hi) where a pass's outputs are needed (the whole grid
// unless the caller needs the closing on part of it only).
struct CBox {
  int lo[3], hi[3];
};
__host__ __device__ __forceinline__ bool cbox_meets(const CBox& b, int x0, int x1, int y0, int y1, int z0, int z1) {
  return x1 >= b.lo[0] && x0 < b.hi[0] && y1 >= b.lo[1] && y0 < b.hi[1] && z1 >= b.lo[2] && z0 < b.hi[2];
}

// The two x-bits of fine row r (y parity r & 1, z parity r >> 1) of four
// packed bytes, gathered into 8 bits (byte b -> bits 2b, 2b+1).
__device__ __forceinline__ uint32_t row_bits8(uint32_t w, int r) {
  uint32_t x = (w >> (2 * r)) & 0x03030303u;
  x = (x | (x >> 6)) & 0x000f000fu;
  return (x | (x >> 12)) & 0xffu;
}

// The four fine rows of 16 packed bytes as 32-bit words (one per row).
__device__ __forceinline__ void rows_of_16_bytes(const uint4 q, uint32_t o[4]) {
#pragma unroll
  for (int r = 0; r < 4; r++)
    o[r] = row_bits8(q.x, r) | (row_bits8(q.y, r) << 8) | (row_bits8(q.z, r) << 16) | (row_bits8(q.w, r) << 24);
}

// ---------------------------------------------------------------------
// pass X of the dilation: 1-D lattice distance to the nearest occupied
// voxel along each fine row, from the packed byte grid.
// ---------------------------------------------------------------------

// One block per packed byte-row (cy, cz), i.e. the four fine rows
// y = 2cy + j, z = 2cz + i.  Shared: 4 rows of N bits (occupied voxels),
// then the corner sets L = bits | bits << 1 (the lattice points that bound
// an occupied voxel), then the nearest set bit of L for every x.
__global__ void __launch_bounds__(256) k_dil_pass_x(const uint8_t* __restrict__ X, uint8_t* __restrict__ A,
                                                    int rx, int ry, int dcap, CBox rows) {
  extern __shared__ uint32_t sm_words[];
  const int N = 2 * rx, Ny = 2 * ry, W = N >> 5;
  const int cy = blockIdx.x, cz = blockIdx.y;
  if (cy < rows.lo[1] || cy >= rows.hi[1] || cz < rows.lo[2] || cz >= rows.hi[2]) return;  // rows nobody reads
  uint32_t* bits = sm_words;            // [4][W]
  uint32_t* corner = sm_words + 4 * W;  // [4][W]
  const uint8_t* row = X + idx3(0, cy, cz, rx, ry);
  // word w of a fine row covers bytes 16w .. 16w+15 of the byte row (W <= 256)
  uint4 q = make_uint4(0u, 0u, 0u, 0u);
  const bool has = threadIdx.x < W;
  if (has) q = *reinterpret_cast<const uint4*>(row + 16 * threadIdx.x);
  const int any = __syncthreads_or(has && (q.x | q.y | q.z | q.w) != 0u);
  const int all = __syncthreads_and(!has || (q.x & q.y & q.z & q.w) == 0xffffffffu);
  if (!any || all) {
    // empty rows: nothing within reach; full rows: every corner is a site
    const uint32_t v = !any ? (uint32_t)dcap * 0x01010101u : 0u;
    const uint4 v4 = make_uint4(v, v, v, v);
    for (int i = threadIdx.x; i < N >> 2; i += blockDim.x) {  // 4 rows x N/16 vectors
      const int r = i / (N >> 4), p16 = 16 * (i - r * (N >> 4));
      *reinterpret_cast<uint4*>(A + idx3(p16, 2 * cy + (r & 1), 2 * cz + (r >> 1), N, Ny)) = v4;
    }
    return;
  }
  if (has) {
    uint32_t o[4];
    rows_of_16_bytes(q, o);
#pragma unroll
    for (int r = 0; r < 4; r++) bits[r * W + threadIdx.x] = o[r];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 4 * W; i += blockDim.x) {
    const int r = i / W, w = i - r * W;
    const uint32_t b = bits[i];
    const uint32_t carry = w > 0 ? bits[r * W + w - 1] >> 31 : 0u;
    corner[i] = b | (b << 1) | carry;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const int r = i / (N >> 2), p4 = 4 * (i - r * (N >> 2));
    const uint32_t* L = corner + r * W;
    uint32_t packed = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int p = p4 + j;
      const int w = p >> 5, b = p & 31;
      int dr = dcap, dl = dcap;
      uint32_t m = L[w] >> b;
      if (m) {
        dr = __ffs(m) - 1;
      } else {
        int acc = 32 - b;
        for (int k = w + 1; k < W && acc < dcap; k++) {
          const uint32_t v = L[k];
          if (v) { acc += __ffs(v) - 1; dr = acc; break; }
          acc += 32;
        }
      }
      m = L[w] << (31 - b);
      if (m) {
        dl = __clz(m);
      } else {
        int acc = b + 1;
        for (int k = w - 1; k >= 0 && acc < dcap; k--) {
          const uint32_t v = L[k];
          if (v) { acc += __clz(v); dl = acc; break; }
          acc += 32;
        }
      }
      int d = dr < dl ? dr : dl;
      if (d > dcap) d = dcap;
      packed |= (uint32_t)d << (8 * j);
    }
    *reinterpret_cast<uint32_t*>(A + idx3(p4, 2 * cy + (r & 1), 2 * cz + (r >> 1), N, Ny)) = packed;
  }
}

// The same pass with one warp per packed byte-row (four fine rows) and no
// shared memory: lane l holds words l, l + 32, .. (WPL per lane) of each
// fine row's corner set, the nearest corner in the words before / after its
// own comes from a warp prefix max / suffix min, and each lane writes the
// 32 distances of each of its words as two 16-byte stores.
constexpr int kBig = 1 << 24;

template <int WPL>
__global__ void __launch_bounds__(256) k_dil_pass_x_w(const uint8_t* __restrict__ X, uint8_t* __restrict__ A,
                                                      int rx, int ry, int rz, int dcap, CBox rows, int64_t row0,
                                                      int64_t row_end) {
  const int lane = threadIdx.x & 31;
  const int64_t row_id = row0 + (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (row_id >= row_end) return;
  const int cy = (int)(row_id % ry), cz = (int)(row_id / ry);
  if (cy < rows.lo[1] || cy >= rows.hi[1] || cz < rows.lo[2] || cz >= rows.hi[2]) return;  // rows nobody reads
  const int N = 2 * rx, Ny = 2 * ry, W = N >> 5;
  const uint8_t* row = X + idx3(0, cy, cz, rx, ry);
  uint32_t L[4][WPL];
  bool any = false, all = true;
#pragma unroll
  for (int k = 0; k < WPL; k++) {
    const int w = lane + 32 * k;
    uint4 q = make_uint4(0u, 0u, 0u, 0u);
    if (w < W) {
      q = *reinterpret_cast<const uint4*>(row + 16 * w);
      all = all && (q.x & q.y & q.z & q.w) == 0xffffffffu;
    }
    any = any || (q.x | q.y | q.z | q.w) != 0u;
    uint32_t o[4];
    rows_of_16_bytes(q, o);
#pragma unroll
    for (int r = 0; r < 4; r++) L[r][k] = o[r];
  }
  any = __any_sync(0xffffffffu, any);
  all = __all_sync(0xffffffffu, all);
  if (!any || all) {
    // empty rows: nothing within reach; full rows: every corner is a site
    const uint32_t v = !any ? (uint32_t)dcap * 0x01010101u : 0u;
    const uint4 v4 = make_uint4(v, v, v, v);
#pragma unroll
    for (int k = 0; k < WPL; k++) {
      const int w = lane + 32 * k;
      if (w >= W) continue;
#pragma unroll
      for (int r = 0; r < 4; r++) {
        uint4* dst = reinterpret_cast<uint4*>(A + idx3(32 * w, 2 * cy + (r & 1), 2 * cz + (r >> 1), N, Ny));
        dst[0] = v4;
        dst[1] = v4;
      }
    }
    return;
  }
#pragma unroll
  for (int r = 0; r < 4; r++) {
    // corner sets: lattice point p bounds voxels p - 1 and p
    uint32_t bits[WPL];
#pragma unroll
    for (int k = 0; k < WPL; k++) bits[k] = L[r][k];
    int first[WPL], last[WPL];
#pragma unroll
    for (int k = 0; k < WPL; k++) {
      // the previous word: lane - 1's, or for lane 0 the last word of the
      // group before (none for word 0)
      uint32_t prev = __shfl_up_sync(0xffffffffu, bits[k], 1);
      const uint32_t tail = k > 0 ? __shfl_sync(0xffffffffu, bits[k > 0 ? k - 1 : 0], 31) : 0u;
      if (lane == 0) prev = tail;
      const uint32_t c = bits[k] | (bits[k] << 1) | (prev >> 31);
      L[r][k] = c;
      const int w = lane + 32 * k;
      first[k] = c ? 32 * w + __ffs(c) - 1 : kBig;
      last[k] = c ? 32 * w + 31 - __clz(c) : -kBig;
    }
    // nearest corner after / before each word
    int nxt[WPL], prv[WPL];
    int after = kBig, before = -kBig;  // over the word groups past / ahead of the current one
#pragma unroll
    for (int k = WPL - 1; k >= 0; k--) {
      int s = first[k];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_down_sync(0xffffffffu, s, o);
        if (lane + o < 32) s = t < s ? t : s;
      }
      int ex = __shfl_down_sync(0xffffffffu, s, 1);
      if (lane == 31) ex = kBig;
      nxt[k] = ex < after ? ex : after;
      const int tot = __shfl_sync(0xffffffffu, s, 0);
      after = tot < after ? tot : after;
    }
#pragma unroll
    for (int k = 0; k < WPL; k++) {
      int s = last[k];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s = t > s ? t : s;
      }
      int ex = __shfl_up_sync(0xffffffffu, s, 1);
      if (lane == 0) ex = -kBig;
      prv[k] = ex > before ? ex : before;
      const int tot = __shfl_sync(0xffffffffu, s, 31);
      before = tot > before ? tot : before;
    }
#pragma unroll
    for (int k = 0; k < WPL; k++) {
      const int w = lane + 32 * k;
      if (w >= W) continue;
      const uint32_t c = L[r][k];
      uint32_t out[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        uint32_t packed = 0;
#pragma unroll
        for (int j4 = 0; j4 < 4; j4++) {
          const int b = 4 * q + j4, pos = 32 * w + b;
          const uint32_t mr = c >> b, ml = c << (31 - b);
          const int dr = mr ? __ffs(mr) - 1 : nxt[k] - pos;
          const int dl = ml ? __clz(ml) : pos - prv[k];
          int d = dr < dl ? dr : dl;
          d = d < dcap ? d : dcap;
          packed |= (uint32_t)d << (8 * j4);
        }
        out[q] = packed;
      }
      uint4* dst = reinterpret_cast<uint4*>(A + idx3(32 * w, 2 * cy + (r & 1), 2 * cz + (r >> 1), N, Ny));
      dst[0] = make_uint4(out[0], out[1], out[2], out[3]);
      dst[1] = make_uint4(out[4], out[5], out[6], out[7]);
    }
  }
}

// launch of the dilation's x pass over the rows of `rows`
static cudaError_t launch_dil_pass_x(const uint8_t* X, uint8_t* A, int rx, int ry, int rz, int dcap, CBox rows,
                                     cudaStream_t st, KernelCounter* kc) {
  const int W = (2 * rx) >> 5;
  // the rows of the box's z range only (row id = y + ry z)
  const int64_t row0 = (int64_t)ry * (rows.lo[2] > 0 ? rows.lo[2] : 0);
  const int64_t row_end = (int64_t)ry * (rows.hi[2] < rz ? rows.hi[2] : rz);
  if (row_end <= row0) return cudaSuccess;
  const unsigned blocks = (unsigned)((row_end - row0 + 7) / 8);
  if (W <= 32) {
    GM_LAUNCH(kc, "k_dil_pass_x", st,
              k_dil_pass_x_w<1><<<blocks, 256, 0, st>>>(X, A, rx, ry, rz, dcap, rows, row0, row_end));
  } else if (W <= 64) {
    GM_LAUNCH(kc, "k_dil_pass_x", st,
              k_dil_pass_x_w<2><<<blocks, 256, 0, st>>>(X, A, rx, ry, rz, dcap, rows, row0, row_end));
  } else {
    GM_LAUNCH(kc, "k_dil_pass_x", st,
              k_dil_pass_x<<<dim3(ry, rz), 256, 8 * W * sizeof(uint32_t), st>>>(X, A, rx, ry, dcap, rows));
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------
// pass X of the erosion: sites are the contour voxels of one fine row;
// outputs the half-voxel-unit partial sums at every voxel centre (HC) and
// at the odd lattice points x = 2c+1 (HL).
// ---------------------------------------------------------------------

// Sites are sparse (the contour shell), so each site splats its
// contribution u(q) + e(q - p)^2 to the outputs within reach with shared
// atomicMin, instead of every output scanning the window.
__global__ void __launch_bounds__(256) k_ero_pass_x(const uint8_t* __restrict__ S, RField R,
                                                    int uniform_r, int rx, int ry, int halo, uint32_t K,
                                                    uint16_t* __restrict__ HC, uint16_t* __restrict__ HL, CBox rows) {
  extern __shared__ uint32_t sm_words[];
  const int res = rx;  // cells along x
  const int N = 2 * rx, Ny = 2 * ry, W = N >> 5;
  const int cy = blockIdx.x, cz = blockIdx.y;
  if (cy < rows.lo[1] || cy >= rows.hi[1] || cz < rows.lo[2] || cz >= rows.hi[2]) return;  // rows nobody reads
  uint32_t* bits = sm_words;              // [4][W]
  uint32_t* hc = sm_words + 4 * W;        // [4][N] centre outputs
  uint32_t* hl = hc + 4 * N;              // [4][res] lattice outputs (x = 2c+1)
  uint32_t* site_pos = hl + 4 * res;      // compacted sites: (row << 16) | x
  uint32_t* site_u = site_pos + 4 * N;    // their offsets K - 4 (r-1)^2
  __shared__ int nsites;
  const uint8_t* row = S + idx3(0, cy, cz, rx, ry);
  if (threadIdx.x == 0) nsites = 0;
  // word w of a fine row covers bytes 16w .. 16w+15 of the byte row (W <= 256)
  uint4 q16 = make_uint4(0u, 0u, 0u, 0u);
  const bool has = threadIdx.x < W;
  if (has) q16 = *reinterpret_cast<const uint4*>(row + 16 * threadIdx.x);
  const int any = __syncthreads_or(has && (q16.x | q16.y | q16.z | q16.w) != 0u);
  if (!any) {
    // no site in these rows: every output keeps the saturation value K
    const uint32_t k2 = K | (K << 16);
    const uint4 v4 = make_uint4(k2, k2, k2, k2);
    for (int i = threadIdx.x; i < N >> 1; i += blockDim.x) {  // 4 rows x N/8 vectors
      const int r = i / (N >> 3), p8 = 8 * (i - r * (N >> 3));
      *reinterpret_cast<uint4*>(HC + idx3(p8, 2 * cy + (r & 1), 2 * cz + (r >> 1), N, Ny)) = v4;
    }
    for (int i = threadIdx.x; i < res >> 1; i += blockDim.x) {  // 4 rows x rx/8 vectors
      const int r = i / (res >> 3), c8 = 8 * (i - r * (res >> 3));
      *reinterpret_cast<uint4*>(HL + idx3(c8, 2 * cy + (r & 1), 2 * cz + (r >> 1), rx, Ny)) = v4;
    }
    return;
  }
  if (has) {
    uint32_t o[4];
    rows_of_16_bytes(q16, o);
#pragma unroll
    for (int r = 0; r < 4; r++) bits[r * W + threadIdx.x] = o[r];
  }
  __syncthreads();
  const int ru = clamp_radius(uniform_r);
  {
    for (int i = threadIdx.x; i < 4 * N; i += blockDim.x) hc[i] = K;
    for (int i = threadIdx.x; i < 4 * res; i += blockDim.x) hl[i] = K;
    // compact the sites with their offsets
    for (int i = threadIdx.x; i < 4 * W; i += blockDim.x) {
      uint32_t m = bits[i];
      if (!m) continue;
      const int r = i / W, w = i - r * W;
      const int base = atomicAdd(&nsites, __popc(m));
      int k = 0;
      while (m) {
        const int x = (w << 5) + __ffs(m) - 1;
        m &= m - 1;
        int rq = ru;
        if (R.p != nullptr) rq = clamp_radius(rget(R, x, 2 * cy + (r & 1), 2 * cz + (r >> 1)));
        site_pos[base + k] = ((uint32_t)r << 16) | (uint32_t)x;
        // offset K - 4 (r-1)^2 (< 2^16) and the site's reach r - 1 (a point
        // at |q - p| >= r(q) is never eroded by q: e >= 2 (r(q) - 1))
        const int reach = rq - 1 < halo ? rq - 1 : halo;
        site_u[base + k] = (K - 4u * (uint32_t)((rq - 1) * (rq - 1))) | ((uint32_t)reach << 16);
        k++;
      }
    }
    __syncthreads();
    const int ns = nsites;
    // one warp per site, lanes over its 2 reach + 1 taps
    const int lane = threadIdx.x & 31;
    for (int sidx = threadIdx.x >> 5; sidx < ns; sidx += blockDim.x >> 5) {
      const uint32_t sp = site_pos[sidx];
      const int r = (int)(sp >> 16), q = (int)(sp & 0xffffu);
      const uint32_t su = site_u[sidx];
      const uint32_t u = su & 0xffffu;
      const int reach = (int)(su >> 16);
      for (int dq = lane - reach; dq <= reach; dq += 32) {
        const int p = q - dq;  // output position, delta = q - p = dq
        if (p < 0 || p >= N) continue;
        const int ec = center_dist2(dq);
        const uint32_t vc = u + (uint32_t)(ec * ec);
        if (vc < K) atomicMin(&hc[r * N + p], vc);
        if (p & 1) {
          const int el = 2 * lattice_dist(dq);
          const uint32_t vl = u + (uint32_t)(el * el);
          if (vl < K) atomicMin(&hl[r * res + (p >> 1)], vl);
        }
      }
    }
    __syncthreads();
  }
  // write out (u16 pairs)
  for (int i = threadIdx.x; i < 2 * N; i += blockDim.x) {
    const int r = i / (N >> 1), p2 = 2 * (i - r * (N >> 1));
    const uint32_t v = hc[r * N + p2] | (hc[r * N + p2 + 1] << 16);
    *reinterpret_cast<uint32_t*>(HC + idx3(p2, 2 * cy + (r & 1), 2 * cz + (r >> 1), N, Ny)) = v;
  }
  for (int i = threadIdx.x; i < 2 * res; i += blockDim.x) {
    const int r = i / (res >> 1), c2 = 2 * (i - r * (res >> 1));
    const uint32_t v = hl[r * res + c2] | (hl[r * res + c2 + 1] << 16);
    *reinterpret_cast<uint32_t*>(HL + idx3(c2, 2 * cy + (r & 1), 2 * cz + (r >> 1), rx, Ny)) = v;
  }
}

// The erosion x pass with one warp per packed byte-row (four fine rows,
// handled one after the other) and no block barrier: the warp's own slice
// of shared memory holds one fine row's outputs (u16) and its site list;
// the warp splats one site at a time, lanes over the site's taps, so the
// lanes of a splat touch distinct outputs and need no atomics.  Rows
// without sites are written as K straight away.  Rows of up to 2048 fine
// voxels (two 32-bit words of sites per lane).
constexpr int kEroXWarps = 8;

__host__ __device__ inline size_t ero_x_w_warp_bytes(int rx) {
  const size_t N = 2 * (size_t)rx;
  return N * 2 + (size_t)rx * 2 + N * 4;  // outputs at centres, at lattice points, sites
}

__global__ void __launch_bounds__(256, 4) k_ero_pass_x_w(const uint8_t* __restrict__ S, RField R, int uniform_r, int rx,
                                                      int ry, int rz, int halo, uint32_t K,
                                                      uint16_t* __restrict__ HC, uint16_t* __restrict__ HL,
                                                      CBox rows) {
  extern __shared__ uint4 sm_ero[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int N = 2 * rx, Ny = 2 * ry, W = N >> 5;
  const int64_t row_id = (int64_t)blockIdx.x * kEroXWarps + wid;
  if (row_id >= (int64_t)ry * rz) return;
  const int cy = (int)(row_id % ry), cz = (int)(row_id / ry);
  if (cy < rows.lo[1] || cy >= rows.hi[1] || cz < rows.lo[2] || cz >= rows.hi[2]) return;  // rows nobody reads
  uint8_t* mine = reinterpret_cast<uint8_t*>(sm_ero) + (size_t)wid * ero_x_w_warp_bytes(rx);
  uint16_t* hc = reinterpret_cast<uint16_t*>(mine);
  uint16_t* hl = reinterpret_cast<uint16_t*>(mine + 2 * (size_t)N);
  uint32_t* sites = reinterpret_cast<uint32_t*>(mine + 2 * (size_t)N + 2 * (size_t)rx);
  const uint8_t* srow = S + idx3(0, cy, cz, rx, ry);
  uint32_t bits[4][2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int w = lane + 32 * k;
    uint4 q = make_uint4(0u, 0u, 0u, 0u);
    if (w < W) q = *reinterpret_cast<const uint4*>(srow + 16 * w);
    uint32_t o[4];
    rows_of_16_bytes(q, o);
#pragma unroll
    for (int r = 0; r < 4; r++) bits[r][k] = o[r];
  }
  const uint32_t k2 = K | (K << 16);
  const uint4 K4 = make_uint4(k2, k2, k2, k2);
  const int ru = clamp_radius(uniform_r);
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const int fy = 2 * cy + (r & 1), fz = 2 * cz + (r >> 1);
    uint4* hcrow = reinterpret_cast<uint4*>(HC + idx3(0, fy, fz, N, Ny));
    uint4* hlrow = reinterpret_cast<uint4*>(HL + idx3(0, fy, fz, rx, Ny));
    const int c = __popc(bits[r][0]) + __popc(bits[r][1]);
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int ns = __shfl_sync(0xffffffffu, incl, 31);
    if (ns == 0) {
      // no site in this row: every output keeps the saturation value K
      for (int i = lane; i < N >> 3; i += 32) hcrow[i] = K4;
      for (int i = lane; i < rx >> 3; i += 32) hlrow[i] = K4;
      continue;
    }
    for (int i = lane; i < N >> 3; i += 32) reinterpret_cast<uint4*>(hc)[i] = K4;
    for (int i = lane; i < rx >> 3; i += 32) reinterpret_cast<uint4*>(hl)[i] = K4;
    // site list: position, r - 1 and reach (a point at |q - p| >= r(q) is
    // never eroded by q: e >= 2 (r(q) - 1))
    int idx = incl - c;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      uint32_t m = bits[r][k];
      while (m) {
        const int x = 32 * (lane + 32 * k) + __ffs(m) - 1;
        m &= m - 1;
        int rq = ru;
        if (R.p != nullptr) rq = clamp_radius(rget(R, x, fy, fz));
        const int reach = rq - 1 < halo ? rq - 1 : halo;
        sites[idx++] = (uint32_t)x | ((uint32_t)(rq - 1) << 12) | ((uint32_t)reach << 20);
      }
    }
    __syncwarp();
    // Runs of adjacent sites with the same radius splat as one: every
    // output inside the run has a site at distance 0 (value u), and one
    // outside it is nearest to the run's end on its side (both kernels grow
    // with the distance), so the run's taps are [q0 - reach, qe + reach]
    // with the nearest site of each, instead of 2 reach + 1 per site.
    for (int i = 0; i < ns;) {
      const uint32_t sw = sites[i];
      const int q0 = (int)(sw & 0xfffu), rm1 = (int)((sw >> 12) & 0xffu), reach = (int)(sw >> 20);
      int j = i + 1;  // first site past the run
      for (;;) {
        const int t = j + lane;
        bool cont = false;
        if (t < ns) {
          const uint32_t st = sites[t];
          cont = (int)(st & 0xfffu) == q0 + (t - i) && (int)((st >> 12) & 0xffu) == rm1;
        }
        const uint32_t brk = __ballot_sync(0xffffffffu, !cont);
        if (brk) {
          j += __ffs(brk) - 1;
          break;
        }
        j += 32;
      }
      const int len = j - i, qe = q0 + len - 1;
      const uint32_t u = K - 4u * (uint32_t)(rm1 * rm1);
      for (int o = lane - reach; o <= len - 1 + reach; o += 32) {
        const int p = q0 + o;  // output position
        if (p < 0 || p >= N) continue;
        const int dq = (o < 0 ? q0 : (o >= len ? qe : p)) - p;  // delta to the nearest site of the run
        const int ec = center_dist2(dq);
        const uint32_t vc = u + (uint32_t)(ec * ec);
        if (vc < K && vc < hc[p]) hc[p] = (uint16_t)vc;
        if (p & 1) {
          const int el = 2 * lattice_dist(dq);
          const uint32_t vl = u + (uint32_t)(el * el);
          if (vl < K && vl < hl[p >> 1]) hl[p >> 1] = (uint16_t)vl;
        }
      }
      __syncwarp();
      i = j;
    }
    for (int i = lane; i < N >> 3; i += 32) hcrow[i] = reinterpret_cast<const uint4*>(hc)[i];
    for (int i = lane; i < rx >> 3; i += 32) hlrow[i] = reinterpret_cast<const uint4*>(hl)[i];
    __syncwarp();
  }
}

// ---------------------------------------------------------------------
// generic axis pass (y or z): out(o) = min over delta of
//     in(pos(o) + delta) (+) g(delta)
// ---------------------------------------------------------------------

enum Kern { KERN_LAT = 0, KERN_LAT2 = 1, KERN_CEN2 = 2, KERN_CUBE = 3 };

template <int G>
__device__ __forceinline__ uint32_t kern_g(int delta) {
  if (G == KERN_LAT) { const int d = lattice_dist(delta); return (uint32_t)(d * d); }
  if (G == KERN_LAT2) { const int d = 2 * lattice_dist(delta); return (uint32_t)(d * d); }
  if (G == KERN_CEN2) { const int d = center_dist2(delta); return (uint32_t)(d * d); }
  return (uint32_t)lattice_dist(delta);  // KERN_CUBE
}

template <int G>
__device__ __forceinline__ uint32_t combine(uint32_t v, uint32_t g) {
  if (G == KERN_CUBE) return v > g ? v : g;
  return v + g;
}

// Minimum over a window of the tile column `col` (stride 32 between
// consecutive positions) around index sp, scanning outward and stopping as
// soon as the kernel alone reaches the best value (inputs are >= 0).
template <int G>
__device__ __forceinline__ uint32_t column_min(const uint16_t* col, int sp, int span, int halo) {
  uint32_t best = combine<G>(col[sp * 32], kern_g<G>(0));
  for (int k = 1; k <= halo; k++) {
    const uint32_t gp = kern_g<G>(k), gm_ = kern_g<G>(-k);
    if ((gp < gm_ ? gp : gm_) >= best) break;
    if (sp + k < span) { const uint32_t v = combine<G>(col[(sp + k) * 32], gp); best = v < best ? v : best; }
    if (sp - k >= 0) { const uint32_t v = combine<G>(col[(sp - k) * 32], gm_); best = v < best ? v : best; }
  }
  return best;
}

constexpr int kTileOut = 64;  // outputs per block along the pass axis
constexpr int kRows = 8;      // blockDim.y

// Input element conversion: u8 fields hold 1-D distances d (pass X of the
// dilation) and enter the sphere kernel squared.
template <int G, typename TIn>
__device__ __forceinline__ uint16_t load_in(const TIn* p, uint32_t cap) {
  const uint32_t v = (uint32_t)*p;
  if (sizeof(TIn) == 1 && G != KERN_CUBE) { const uint32_t s = v * v; return (uint16_t)(s < cap ? s : cap); }
  return (uint16_t)(v < cap ? v : cap);
}

// in/out fields are x-fastest with dims (nx, ny, nz).  axis = 1 (y) or 2
// (z).  sub: output only the odd input positions 2o+1 along the axis.
template <int G, typename TIn>
__global__ void __launch_bounds__(256) k_axis_pass(const TIn* __restrict__ in, uint16_t* __restrict__ out,
                                                   int nx, int ny, int nz, int axis, int sub, int halo,
                                                   uint32_t cap) {
  extern __shared__ uint16_t tile[];  // [span][32]
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = blockIdx.x * 32 + tx;
  const int na = axis == 1 ? ny : nz;
  const int nout = sub ? na / 2 : na;
  const int third = blockIdx.z;  // z for axis y, y for axis z
  const int64_t sa = axis == 1 ? (int64_t)nx : (int64_t)nx * ny;
  const int64_t s3 = axis == 1 ? (int64_t)nx * ny : (int64_t)nx;
  const int o0 = blockIdx.y * kTileOut;
  const int p_first = sub ? 2 * o0 + 1 : o0;
  const int o_last = min(o0 + kTileOut, nout) - 1;
  const int p_last = sub ? 2 * o_last + 1 : o_last;
  const int lo = p_first - halo;
  const int span = p_last + halo - lo + 1;
  for (int s = ty; s < span; s += kRows) {
    const int a = lo + s;
    uint16_t v = (uint16_t)cap;
    if (x < nx && a >= 0 && a < na) v = load_in<G, TIn>(in + x + sa * a + s3 * third, cap);
    tile[s * 32 + tx] = v;
  }
  __syncthreads();
  if (x >= nx) return;
  // output dims: same as input except the pass axis (nout)
  const int64_t osa = sa;
  const int64_t os3 = axis == 1 ? (int64_t)nx * nout : (int64_t)nx;
  for (int o = o0 + ty; o <= o_last; o += kRows) {
    const int p = sub ? 2 * o + 1 : o;
    const uint32_t best = column_min<G>(tile + tx, p - lo, span, halo);
    out[x + osa * o + os3 * third] = (uint16_t)(best < cap ? best : cap);
  }
}

// ---------------------------------------------------------------------
// final z pass at full resolution, fused with the per-voxel threshold and
// the packing of 2x2x2 bits into reference bytes.
//   FIN_DIL: bit = sum < (r(p)+1)^2 (sphere) / sum <= r(p) (cube)
//   FIN_ERO: bit = sum < K (eroded)
// block (32, 8): tx = x, ty & 1 = y parity, ty >> 1 = group of 16 z.
// ---------------------------------------------------------------------

enum Fin { FIN_DIL = 0, FIN_ERO = 1 };

template <int G, int F>
__global__ void __launch_bounds__(256) k_final_z(const uint16_t* __restrict__ in, uint8_t* __restrict__ out_cells,
                                                 RField R, int uniform_r, int rx, int ry, int rz,
                                                 int halo, uint32_t cap) {
  extern __shared__ uint16_t tile2[];  // [2][span][32]
  const int Nx = 2 * rx, Ny = 2 * ry, N = 2 * rz;  // N: fine extent along the pass axis z
  const int tx = threadIdx.x, yp = threadIdx.y & 1, zg = threadIdx.y >> 1;
  const int x = blockIdx.x * 32 + tx;
  const int y = 2 * blockIdx.z + yp;
  const int z0 = blockIdx.y * kTileOut;
  const int z_last = min(z0 + kTileOut, N) - 1;
  const int lo = z0 - halo;
  const int span = z_last + halo - lo + 1;
  uint16_t* tile = tile2 + yp * span * 32;
  for (int s = zg; s < span; s += 4) {
    const int a = lo + s;
    uint16_t v = (uint16_t)cap;
    if (x < Nx && a >= 0 && a < N) {
      const uint32_t t = in[idx3(x, y, a, Nx, Ny)];
      v = (uint16_t)(t < cap ? t : cap);
    }
    tile[s * 32 + tx] = v;
  }
  __syncthreads();
  // each thread: 16 consecutive z = z0 + 16 zg + j
  uint32_t bits = 0;
  const int ru = clamp_radius(uniform_r);
  if (x < Nx) {
#pragma unroll 1
    for (int j = 0; j < 16; j++) {
      const int z = z0 + 16 * zg + j;
      if (z > z_last) break;
      const uint32_t v = column_min<G>(tile + tx, z - lo, span, halo);
      bool b;
      if (F == FIN_DIL) {
        const int r = R.p != nullptr ? clamp_radius(rget(R, x, y, z)) : ru;
        if (G == KERN_CUBE) b = v <= (uint32_t)r;
        else b = v < (uint32_t)((r + 1) * (r + 1));
      } else {
        b = v < cap;
      }
      bits |= (uint32_t)b << j;
    }
  }
  // pack: for z pair q (0..7), this voxel contributes bit (xb + 2 yb) for the
  // lower z and (xb + 2 yb + 4) for the upper z.
  const int xb = x & 1;
  uint32_t packed = 0;  // byte q in bits 8q..8q+7, q = 0..3 (first 8 z) / second word
  uint32_t packed_hi = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const uint32_t lo_b = (bits >> (2 * q)) & 1u, hi_b = (bits >> (2 * q + 1)) & 1u;
    const uint32_t byte = (lo_b << (xb + 2 * yp)) | (hi_b << (xb + 2 * yp + 4));
    if (q < 4) packed |= byte << (8 * q);
    else packed_hi |= byte << (8 * (q - 4));
  }
  packed |= __shfl_xor_sync(0xffffffffu, packed, 1);
  packed_hi |= __shfl_xor_sync(0xffffffffu, packed_hi, 1);
  __shared__ uint32_t ex[2][4][32][2];
  ex[yp][zg][tx][0] = packed;
  ex[yp][zg][tx][1] = packed_hi;
  __syncthreads();
  if (yp == 0 && (tx & 1) == 0 && x < Nx) {
    const uint32_t w0 = packed | ex[1][zg][tx][0];
    const uint32_t w1 = packed_hi | ex[1][zg][tx][1];
    const int cx = x >> 1, cyy = y >> 1;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int zc = (z0 + 16 * zg) / 2 + q;
      if (2 * zc > z_last) break;
      const uint32_t byte = q < 4 ? (w0 >> (8 * q)) & 0xffu : (w1 >> (8 * (q - 4))) & 0xffu;
      out_cells[idx3(cx, cyy, zc, rx, ry)] = (uint8_t)byte;
    }
  }
}

// final z pass of the base erosion: lattice points 2c+1 only; one flag byte
// per base cell (1 = the cell centre is eroded).
__global__ void __launch_bounds__(256) k_final_z_base(const uint16_t* __restrict__ in, uint8_t* __restrict__ flags,
                                                      int rx, int ry, int rz, int halo, uint32_t cap) {
  extern __shared__ uint16_t tile[];
  const int N = 2 * rz;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = blockIdx.x * 32 + tx;  // cx
  const int cyy = blockIdx.z;
  const int o0 = blockIdx.y * kTileOut;
  const int o_last = min(o0 + kTileOut, rz) - 1;
  const int lo = 2 * o0 + 1 - halo;
  const int span = 2 * o_last + 1 + halo - lo + 1;
  for (int s = ty; s < span; s += kRows) {
    const int a = lo + s;
    uint16_t v = (uint16_t)cap;
    if (x < rx && a >= 0 && a < N) {
      const uint32_t t = in[idx3(x, cyy, a, rx, ry)];
      v = (uint16_t)(t < cap ? t : cap);
    }
    tile[s * 32 + tx] = v;
  }
  __syncthreads();
  if (x >= rx) return;
  for (int o = o0 + ty; o <= o_last; o += kRows) {
    const uint32_t v = column_min<KERN_LAT2>(tile + tx, 2 * o + 1 - lo, span, halo);
    flags[idx3(x, cyy, o, rx, ry)] = v < cap ? 1 : 0;
  }
}

// ---------------------------------------------------------------------
// packed 16-bit min-plus pass (y or z) with DPX add-min
//
// Each thread owns two adjacent x columns (one u32 = two u16 lanes) and 16
// consecutive outputs along the pass axis, so one __viaddmin_u16x2 updates
// two outputs per tap.  A block is 64 columns x 64 outputs x 2 "third"
// coordinates (256 threads); the input tile with its halo sits in shared
// memory.  Taps are visited outward (|delta| = 0, 1, 2, ...); a warp stops
// as soon as the kernel alone exceeds every output it holds.  A tile with
// no finite input is written directly.  Requires cap <= 32767 so that
// value + kernel never wraps in 16 bits.
//   FIN 0: write the u16 field;  FIN 1: dilation threshold + packed bytes;
//   FIN 2: erosion threshold (centres) + packed bytes;
//   FIN 3: erosion threshold at lattice points 2c+1, one flag per cell.
// ---------------------------------------------------------------------

constexpr int kDpxCols = 64;   // x columns per block
constexpr int kDpxOut = 64;    // outputs per block along the axis (4 warps x 16)
constexpr int kDpxPer = 16;    // outputs per thread

template <int G>
__device__ __forceinline__ uint32_t gpair(int delta, uint32_t cap) {
  uint32_t g = kern_g<G>(delta);
  g = g < cap ? g : cap;
  return g | (g << 16);
}

// kernel value at delta = k >= 1 (the +side), without the general
// lattice_dist; the -side of LAT and CUBE at -k equals the +side at k - 1,
// and CEN2 is symmetric
template <int G>
__device__ __forceinline__ uint32_t kern_pos(int k) {
  if (G == KERN_LAT) return (uint32_t)(k * k);
  if (G == KERN_LAT2) return (uint32_t)(4 * k * k);
  if (G == KERN_CEN2) return (uint32_t)((2 * k - 1) * (2 * k - 1));
  return (uint32_t)k;  // KERN_CUBE
}

__device__ __forceinline__ uint32_t pack_cap(uint32_t g, uint32_t cap) {
  g = g < cap ? g : cap;
  return g | (g << 16);
}

template <int G>
__device__ __forceinline__ uint32_t step_min(uint32_t row, uint32_t g, uint32_t best) {
  if (G == KERN_CUBE) return __vminu2(__vmaxu2(row, g), best);
  return __viaddmin_u16x2(row, g, best);
}

template <int G, typename TIn>
__device__ __forceinline__ uint32_t load_pair(const TIn* p, uint32_t capp) {
  uint32_t v;
  if (sizeof(TIn) == 1) {
    const uint32_t w = *reinterpret_cast<const uint16_t*>(p);
    const uint32_t a = w & 0xffu, b = w >> 8;
    v = G != KERN_CUBE ? (a * a) | ((b * b) << 16) : a | (b << 16);
  } else {
    v = *reinterpret_cast<const uint32_t*>(p);
  }
  return __vminu2(v, capp);  // both lanes saturated at cap
}

size_t dpx_smem_bytes(int sub, int halo) {
  const int span = (sub ? 2 * kDpxOut - 1 : kDpxOut) + 2 * halo;
  return (size_t)2 * span * 32 * sizeof(uint32_t) + 128;  // + slack to align the tile to 128 bytes (TMA)
}

// Where a pass's outputs are needed: tiles whose cells, grown by (gx, ga,
// gt) cells along (x, pass axis, third axis), hold no non-empty cell of the
// 8^3-cell occupancy map of the dilation are skipped.  The x coordinate and
// the third coordinate are fine voxels (shift 1) or cells (shift 0); the
// outputs along the pass axis are fine voxels (sub = 0) or cells (sub = 1).
struct NeedMap {
  const uint8_t* dmap;  // nullptr: no occupancy test
  int mdx, mdy, mdz;
  int x_shift, t_shift;
  int gx, ga, gt;
  CBox roi;             // tiles whose own cells miss it are skipped as well
  // launch over third-axis block rows third0 .. third0 + third_n - 1 and
  // output tiles out0 .. out0 + out_n - 1 only (0: all); a skipped tile
  // writes saturation values, so a part of a pass that must leave the rest
  // of its output alone is launched this way
  int third0 = 0, third_n = 0, out0 = 0, out_n = 0;
};

__device__ bool tile_needed(const NeedMap& nm, int axis, int sub, int o0, int nout, int bx, int bz) {
  const int x0 = bx * kDpxCols;
  const int cx0 = x0 >> nm.x_shift, cx1 = (x0 + kDpxCols - 1) >> nm.x_shift;
  const int oa = o0, ob = min(o0 + kDpxOut, nout) - 1;
  const int ca0 = sub ? oa : oa >> 1, ca1 = sub ? ob : ob >> 1;
  const int ct0 = (2 * bz) >> nm.t_shift, ct1 = (2 * bz + 1) >> nm.t_shift;
  // (a, t) are (y, z) for the y pass and (z, y) for the z pass
  {
    const int ya = axis == 1 ? ca0 : ct0, yb = axis == 1 ? ca1 : ct1;
    const int za = axis == 1 ? ct0 : ca0, zb = axis == 1 ? ct1 : ca1;
    if (!cbox_meets(nm.roi, cx0, cx1, ya, yb, za, zb)) return false;  // block-uniform
  }
  if (nm.dmap == nullptr) return true;
  const int lo[3] = {cx0 - nm.gx, (axis == 1 ? ca0 - nm.ga : ct0 - nm.gt), (axis == 1 ? ct0 - nm.gt : ca0 - nm.ga)};
  const int hi[3] = {cx1 + nm.gx, (axis == 1 ? ca1 + nm.ga : ct1 + nm.gt), (axis == 1 ? ct1 + nm.gt : ca1 + nm.ga)};
  const int md[3] = {nm.mdx, nm.mdy, nm.mdz};
  int a[3], b[3], c[3];
  for (int k = 0; k < 3; k++) {
    a[k] = max(lo[k], 0) >> 3;
    b[k] = min(hi[k] >> 3, md[k] - 1);
    c[k] = b[k] - a[k] + 1;
  }
  int any = 0;
  if (c[0] > 0 && c[1] > 0 && c[2] > 0)
    for (int i = threadIdx.x; i < c[0] * c[1] * c[2]; i += blockDim.x) {
      const int ix = a[0] + i % c[0], iy = a[1] + (i / c[0]) % c[1], iz = a[2] + i / (c[0] * c[1]);
      any |= nm.dmap[idx3(ix, iy, iz, nm.mdx, nm.mdy)];
    }
  return __syncthreads_or(any) != 0;
}

// Radius bound of one tile of a dilation pass, from the map of the largest
// raw radius per 16^3 fine voxels: over the tile's x columns and outputs,
// and its two third-axis coordinates widened by `rext` (the y pass feeds z
// outputs up to a halo away).  Block-uniform.
__device__ int tile_radius(const uint8_t* __restrict__ rmap, int mbx, int mby, int nx, int n3, int axis, int nout,
                           int o0, int rext, int bx, int bz) {
  __shared__ int rt_s;
  if (threadIdx.x == 0) rt_s = 0;
  __syncthreads();
  const int xa = (bx * kDpxCols) >> 4, xb = (min(bx * kDpxCols + kDpxCols, nx) - 1) >> 4;
  const int aa = o0 >> 4, ab = (min(o0 + kDpxOut, nout) - 1) >> 4;
  const int ta = max(2 * bz - rext, 0) >> 4, tb = min(2 * bz + 1 + rext, n3 - 1) >> 4;
  const int cx = xb - xa + 1, ca = ab - aa + 1, ct = tb - ta + 1;
  int m = 0;
  for (int i = threadIdx.x; i < cx * ca * ct; i += blockDim.x) {
    const int ix = xa + i % cx, ia = aa + (i / cx) % ca, it = ta + i / (cx * ca);
    const int my = axis == 1 ? ia : it, mz = axis == 1 ? it : ia;
    const int v = rmap[idx3(ix, my, mz, mbx, mby)];
    m = v > m ? v : m;
  }
  for (int o = 16; o > 0; o >>= 1) { const int t = __shfl_xor_sync(0xffffffffu, m, o); m = t > m ? t : m; }
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(&rt_s, m);
  __syncthreads();
  return clamp_radius(rt_s);
}

// One tile of a min-plus pass: 64 columns x 64 outputs x 2 third-axis
// slices, at tile coordinates (bx, by, bz) along (x, outputs, slice pairs),
// the need map's out0 / third0 offsets included.  The whole block works on
// it.  With use_tma, the u16 input tile is staged by TMA (tmap: boxes of 64
// columns x span rows x 1 slice along (x, pass axis, third axis), one per
// slice; rows are 128 bytes, so each slice starts 128-byte aligned).
template <int G, typename TIn, int FIN>
__device__ __forceinline__ void dpx_tile(const TIn* __restrict__ in, uint16_t* __restrict__ out16,
                                         uint8_t* __restrict__ out8, int nx, int ny, int nz, int axis, int sub,
                                         int halo, uint32_t cap, RField R, int uniform_r, int rx, int ry,
                                         const uint8_t* __restrict__ rmap, int rext, const NeedMap& need,
                                         const CUtensorMap* tmap, int use_tma, int bx, int by, int bz) {
  extern __shared__ uint32_t tile_raw[];
  uint32_t* tileu = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(tile_raw) + 127) & ~(uintptr_t)127);
  __shared__ uint64_t tma_bar;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tpar = w >> 2, grp = w & 3;
  const int x = bx * kDpxCols + 2 * lane;
  const int na = axis == 1 ? ny : nz;
  const int n3 = axis == 1 ? nz : ny;
  const int nout = sub ? na / 2 : na;
  const int third = 2 * bz + tpar;
  const int64_t sa = axis == 1 ? (int64_t)nx : (int64_t)nx * ny;
  const int64_t s3 = axis == 1 ? (int64_t)nx * ny : (int64_t)nx;
  const int o0 = by * kDpxOut;
  const int step = sub ? 2 : 1;
  const int lo = (sub ? 2 * o0 + 1 : o0) - halo;
  const int span = (sub ? 2 * kDpxOut - 1 : kDpxOut) + 2 * halo;
  // Dilation passes with a radius field use the tile's own radius bound:
  // a smaller window (halo_e) and saturation value (cap_e).  Every output
  // that reads this tile has r(p) <= rt, so terms >= (rt+1)^2 never decide.
  int halo_e = halo;
  if (rmap != nullptr && step == 1) {
    const int rt = tile_radius(rmap, nx >> 4, ny >> 4, nx, n3, axis, nout, o0, rext, bx, bz);
    const uint32_t ct = G == KERN_CUBE ? (uint32_t)(rt + 1) : (uint32_t)((rt + 1) * (rt + 1));
    cap = ct < cap ? ct : cap;
    halo_e = rt + 2 < halo ? rt + 2 : halo;
  }
  // Erosion outputs matter only where the dilation has voxels (and the
  // passes feeding them within their window): a tile outside writes its
  // saturation value ("not eroded") without work.
  const bool needed = tile_needed(need, axis, sub, o0, nout, bx, bz);
  const int skip = needed ? halo - halo_e : span;  // tile rows never read
  const uint32_t capp = cap | (cap << 16);
  const int tile_rows = span;
  uint32_t* tile = tileu + tpar * tile_rows * 32;
  const bool colok = x < nx && third < n3;
  int finite = 0;
  constexpr bool kTileMin = G == KERN_CEN2 || G == KERN_LAT2 || (G == KERN_LAT && FIN == 1);
  uint32_t vmin = 0xffffffffu;  // smallest loaded value (both lanes)
  // TMA staging (u16 inputs): the whole span of both slices, one copy per
  // slice issued by one thread; rows past the field come back as zeros and
  // are set to the saturation value below, with the rows [skip, span - skip)
  // that the taps read.
  const int nchunks = sizeof(TIn) == 2 && use_tma && span - 2 * skip > 0 ? 1 : 0;  // block-uniform
  if (nchunks > 0) {
    if (threadIdx.x == 0) {
      tma_prefetch_map(tmap);
      mbar_init(&tma_bar, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_arrive_expect_tx(&tma_bar, (uint32_t)(2 * span * kDpxCols * sizeof(uint16_t)));
      const int x0 = bx * kDpxCols, t0 = 2 * bz;
      for (int tp = 0; tp < 2; tp++) {
        uint32_t* dst = tileu + tp * tile_rows * 32;
        if (axis == 1)
          tma_load_3d(dst, tmap, x0, lo, t0 + tp, &tma_bar);
        else
          tma_load_3d(dst, tmap, x0, t0 + tp, lo, &tma_bar);
      }
    }
    if (!mbar_wait_bounded(&tma_bar, 0, 1u << 22)) atomicOr(&g_kernel_errors, kErrTmaTimeout);
  }
  for (int s = skip + grp; s < span - skip; s += 4) {
    const int a = lo + s;
    uint32_t v = capp;
    if (colok && a >= 0 && a < na)
      v = nchunks > 0 ? __vminu2(tile[s * 32 + lane], capp) : load_pair<G, TIn>(in + x + sa * a + s3 * third, capp);
    tile[s * 32 + lane] = v;
    finite |= v != capp;
    if (kTileMin) vmin = __vminu2(vmin, v);
  }
  __shared__ uint32_t warp_min[8];
  if (kTileMin) {
    const uint32_t m2 = (vmin & 0xffffu) < (vmin >> 16) ? (vmin & 0xffffu) : (vmin >> 16);
    const uint32_t mw = __reduce_min_sync(0xffffffffu, m2);
    if (lane == 0) warp_min[w] = mw;
  }
  finite = __syncthreads_or(finite);
  // Every tile value is >= tmin, so a tap whose kernel value reaches
  // cap - tmin cannot bring an output below the saturation value cap: the
  // window of this tile ends at the last tap below it (kernels grow with
  // |delta|).  Erosion passes: their inputs carry the per-site offset
  // K - 4 (r - 1)^2, so tiles whose sites all have small radii need short
  // windows; the final dilation pass: tiles whose inputs are all far from
  // the input stop early.  (The first dilation pass, whose tiles next to a
  // surface hold zeros, is faster without it.)
  uint32_t tmin = 0;
  int halo_t = step == 1 ? halo_e : halo;
  if (kTileMin) {
    tmin = warp_min[0];
#pragma unroll
    for (int i = 1; i < 8; i++) tmin = warp_min[i] < tmin ? warp_min[i] : tmin;
  }
  if (kTileMin && finite) {
    int hm = 1;
    while (hm < halo_t && (step == 1 ? kern_pos<G>(hm)
                                     : (kern_g<G>(hm) < kern_g<G>(-hm) ? kern_g<G>(hm) : kern_g<G>(-hm))) +
                                  tmin < cap)
      hm++;
    halo_t = hm < halo_t ? hm : halo_t;
  }
  const int obase = o0 + grp * kDpxPer;
  const int sp0 = (sub ? 2 * obase + 1 : obase) - lo;
  uint32_t best[kDpxPer];
  // The lattice-point erosion (KERN_LAT2) is the only pass with outputs at
  // every other position (sub, step 2) and the only one that has them:
  // each instantiation compiles one of the two tap loops.
  constexpr bool kSub = G == KERN_LAT2;
  if (finite && !kSub) {
    // Register sliding windows: wp[(j + k) % 16] holds tile row sp0 + j + k
    // and wm[(j - k) mod 16] holds row sp0 + j - k, so that after tap k only
    // one new row per side is loaded (into the slot its leaving row frees).
    // Rows read: sp0 - halo_t .. sp0 + 15 + halo_t (halo_t <= halo_e, and
    // at least the rows sp0 - 1 and sp0 + 16 of the first window), inside
    // [skip, span - skip).
    const uint32_t* tcol = tile + lane;
    uint32_t wp[kDpxPer], wm[kDpxPer];
#pragma unroll
    for (int j = 0; j < kDpxPer; j++) {
      wp[j] = tcol[(sp0 + j + (j < 1 ? kDpxPer : 0)) * 32];
      wm[j] = tcol[(sp0 + (j < kDpxPer - 1 ? j : -1)) * 32];
    }
    const uint32_t g0 = gpair<G>(0, cap);
#pragma unroll
    for (int j = 0; j < kDpxPer; j++) best[j] = step_min<G>(tcol[(sp0 + j) * 32], g0, capp);
    uint32_t gprev = g0;  // +side kernel of the previous tap (the -side of this one for LAT, CUBE)
    for (int kb = 0; kb <= halo_t; kb += kDpxPer) {
#pragma unroll
      for (int u = 0; u < kDpxPer; u++) {
        const int k = kb + u;
        if (k == 0) continue;
        if (k > halo_t) goto dpx_done;
        const uint32_t graw = kern_pos<G>(k);
        const uint32_t gp = pack_cap(graw, cap);
        const uint32_t gm_ = G == KERN_CEN2 ? gp : gprev;
        gprev = gp;
#pragma unroll
        for (int j = 0; j < kDpxPer; j++) {
          best[j] = step_min<G>(wp[(j + u) % kDpxPer], gp, best[j]);
          best[j] = step_min<G>(wm[(j - u + kDpxPer) % kDpxPer], gm_, best[j]);
        }
        if (k == halo_t) goto dpx_done;  // no further tap: load nothing past the window
        // rows sp0 + k + 16 and sp0 - k - 1 enter; the slots of rows
        // sp0 + k and sp0 + 15 - k are free now (k < halo_e keeps both in the window)
        wp[u] = tcol[(sp0 + k + kDpxPer) * 32];
        wm[(kDpxPer - 1 - u) % kDpxPer] = tcol[(sp0 - k - 1) * 32];
        if ((u & 3) == 3) {  // every fourth tap: leave once no output can improve
          uint32_t m = best[0];
#pragma unroll
          for (int j = 1; j < kDpxPer; j++) m = __vmaxu2(m, best[j]);
          const uint32_t mx = (m & 0xffffu) > (m >> 16) ? (m & 0xffffu) : (m >> 16);
          // smallest kernel value of the taps to come (k + 1 on either side)
          const uint32_t nxt = G == KERN_CEN2 ? kern_pos<G>(k + 1) : graw;
          if (__all_sync(0xffffffffu, nxt + tmin >= mx)) goto dpx_done;
        }
      }
    }
  dpx_done:;
  } else if (finite && kSub) {
    // Outputs at every other position (sub): output j sits on tile row
    // sp0 + 2j and reads rows sp0 + 2j + delta.  The taps split by the
    // parity of delta into two stride-1 sequences over the rows of one
    // parity, R(h) = row b + 2h (b = sp0: delta = 2d; b = sp0 - 1:
    // delta = 2d - 1; h = j + d), each run with the register sliding window
    // of the full-resolution path: one new row per side and tap instead of
    // one load per output and tap.
#pragma unroll
    for (int j = 0; j < kDpxPer; j++) best[j] = capp;
    const uint32_t* tcol = tile + lane;
#pragma unroll 1
    for (int par = 0; par < 2; par++) {
      const int e0 = -par;                   // delta of the group's centre tap (d = 0)
      const uint32_t* tb = tcol + (sp0 - par) * 32;  // R(h) = tb[64 h]
      const int kp = (halo_t - e0) >> 1;     // plus taps d = k: delta = 2k + e0 <= halo_t
      const int km = (halo_t + e0) >> 1;     // minus taps d = -k: delta = -2k + e0 >= -halo_t
      const int kmax = kp > km ? kp : km;
      uint32_t wp[kDpxPer], wm[kDpxPer];
#pragma unroll
      for (int j = 0; j < kDpxPer; j++) {
        wp[j] = tb[(j < 1 ? kDpxPer : j) * 64];
        wm[j] = tb[(j < kDpxPer - 1 ? j : -1) * 64];
      }
      const uint32_t gc = pack_cap(kern_g<G>(e0), cap);
#pragma unroll
      for (int j = 0; j < kDpxPer; j++) best[j] = step_min<G>(tb[j * 64], gc, best[j]);
      for (int kb = 0; kb <= kmax; kb += kDpxPer) {
#pragma unroll
        for (int u = 0; u < kDpxPer; u++) {
          const int k = kb + u;
          if (k == 0) continue;
          if (k > kmax) goto sub_done;
          if (k <= kp) {
            const uint32_t gp = pack_cap(kern_g<G>(2 * k + e0), cap);
#pragma unroll
            for (int j = 0; j < kDpxPer; j++) best[j] = step_min<G>(wp[(j + u) % kDpxPer], gp, best[j]);
          }
          if (k <= km) {
            const uint32_t gm_ = pack_cap(kern_g<G>(-2 * k + e0), cap);
#pragma unroll
            for (int j = 0; j < kDpxPer; j++)
              best[j] = step_min<G>(wm[(j - u + kDpxPer) % kDpxPer], gm_, best[j]);
          }
          if (k == kmax) goto sub_done;
          // R(k + 16) and R(-k - 1) enter for the next tap, in the slots
          // that R(k) and R(15 - k) leave
          if (k < kp) wp[u] = tb[(k + kDpxPer) * 64];
          if (k < km) wm[(kDpxPer - 1 - u) % kDpxPer] = tb[(-k - 1) * 64];
          if ((u & 3) == 3) {  // every fourth tap: leave once no output can improve
            uint32_t m = best[0];
#pragma unroll
            for (int j = 1; j < kDpxPer; j++) m = __vmaxu2(m, best[j]);
            const uint32_t mx = (m & 0xffffu) > (m >> 16) ? (m & 0xffffu) : (m >> 16);
            const uint32_t np = k + 1 <= kp ? kern_g<G>(2 * (k + 1) + e0) : 0xffffu;
            const uint32_t nm = k + 1 <= km ? kern_g<G>(-2 * (k + 1) + e0) : 0xffffu;
            const uint32_t nxt = np < nm ? np : nm;
            if (__all_sync(0xffffffffu, nxt + tmin >= mx)) goto sub_done;
          }
        }
      }
    sub_done:;
    }
  } else {
#pragma unroll
    for (int j = 0; j < kDpxPer; j++) best[j] = capp;
  }
  if (FIN == 0) {
    if (!colok) return;
    const int64_t osa = axis == 1 ? (int64_t)nx : (int64_t)nx * ny;
    const int64_t os3 = axis == 1 ? (int64_t)nx * nout : (int64_t)nx;
#pragma unroll
    for (int j = 0; j < kDpxPer; j++) {
      const int o = obase + j;
      if (o < nout) *reinterpret_cast<uint32_t*>(out16 + x + osa * o + os3 * third) = best[j];
    }
  } else if (FIN == 3) {
    if (!colok) return;
    // x is a cell index here; outputs are cells (x, third, o)
#pragma unroll
    for (int j = 0; j < kDpxPer; j++) {
      const int o = obase + j;
      if (o >= nout) continue;
      const uint32_t v = best[j];
      uint8_t* dst = out8 + idx3(x, third, o, rx, ry);
      dst[0] = (v & 0xffffu) < cap ? 1 : 0;
      dst[1] = (v >> 16) < cap ? 1 : 0;
    }
  } else {
    // threshold then pack 2 (x) x 2 (y = third pair) x 2 (z) bits per byte
    __shared__ uint32_t xch[4][32][2];
    const int N = nz;  // fine extent along the pass axis (z)
    const int ru = clamp_radius(uniform_r);
    uint32_t bytes[2] = {0u, 0u};  // 8 z pairs: bytes q = 0..7
#pragma unroll
    for (int j = 0; j < kDpxPer; j++) {
      const int z = obase + j;
      const uint32_t v = best[j];
      // per-lane thresholds T (bit = value < T)
      uint32_t tpair;
      if (FIN == 1) {
        uint32_t r2;  // the two clamped radii, one per u16 lane
        if (R.p != nullptr && colok && z < N) {
          // x even and even strides: a 2-byte aligned pair
          const uint32_t rr = *reinterpret_cast<const uint16_t*>(R.p + (int64_t)x + third * R.sy + z * R.sz);
          const uint32_t c = __vmins4(__vmaxs4(rr, 0x02020202u), 0x7f7f7f7fu);  // clamp to [2, 127] per byte
          r2 = __byte_perm(c, 0u, 0x4140);
        } else {
          r2 = (uint32_t)ru | ((uint32_t)ru << 16);
        }
        const uint32_t r1 = r2 + 0x00010001u;  // r + 1 per lane (<= 128)
        if (G == KERN_CUBE) {
          tpair = r1;  // value <= r
        } else {
          const uint32_t lo = r1 & 0xffffu, hi = r1 >> 16;
          tpair = (lo * lo) | ((hi * hi) << 16);  // value < (r + 1)^2
        }
      } else {
        tpair = capp;
      }
      const uint32_t m = __vcmpltu2(v, tpair);  // 0xffff per lane below its threshold
      const uint32_t b2 = (m & 1u) | ((m >> 15) & 2u);
      const int q = j >> 1, zb = j & 1;
      bytes[q >> 2] |= (b2 << (2 * tpar + 4 * zb)) << (8 * (q & 3));
    }
    if (tpar == 1) {
      xch[grp][lane][0] = bytes[0];
      xch[grp][lane][1] = bytes[1];
    }
    __syncthreads();
    if (tpar == 0 && colok) {
      bytes[0] |= xch[grp][lane][0];
      bytes[1] |= xch[grp][lane][1];
      const int cx = x >> 1, cy = third >> 1;
#pragma unroll
      for (int q = 0; q < kDpxPer / 2; q++) {
        const int cz = obase / 2 + q;
        if (2 * cz < N) out8[idx3(cx, cy, cz, rx, ry)] = (uint8_t)((bytes[q >> 2] >> (8 * (q & 3))) & 0xffu);
      }
    }
  }
}

template <int G, typename TIn, int FIN>
__global__ void __launch_bounds__(256, 4) k_pass_dpx(const TIn* __restrict__ in, uint16_t* __restrict__ out16,
                                                  uint8_t* __restrict__ out8, int nx, int ny, int nz, int axis,
                                                  int sub, int halo, uint32_t cap, RField R,
                                                  int uniform_r, int rx, int ry, const uint8_t* __restrict__ rmap,
                                                  int rext, NeedMap need, const __grid_constant__ CUtensorMap tmap,
                                                  int use_tma) {
  dpx_tile<G, TIn, FIN>(in, out16, out8, nx, ny, nz, axis, sub, halo, cap, R, uniform_r, rx, ry, rmap, rext, need,
                        &tmap, use_tma, (int)blockIdx.x, (int)blockIdx.y + need.out0, (int)blockIdx.z + need.third0);
}

template <int G, typename TIn, int FIN>
static void launch_dpx(const TIn* in, uint16_t* out16, uint8_t* out8, int nx, int ny, int nz, int axis, int sub,
                       int halo, uint32_t cap, RField R, int uniform_r, int rx, int ry, cudaStream_t st,
                       KernelCounter* kc, const char* name, const uint8_t* rmap = nullptr, int rext = 0,
                       NeedMap need = NeedMap{nullptr, 0, 0, 0, 0, 0, 0, 0, 0, CBox{{0, 0, 0}, {1 << 30, 1 << 30, 1 << 30}}}) {
  if ((G == KERN_LAT2) != (sub != 0)) return;  // (every call site pairs them; see k_pass_dpx)
  const size_t smem = dpx_smem_bytes(sub, halo);
  ensure_dynamic_smem(reinterpret_cast<const void*>(k_pass_dpx<G, TIn, FIN>), smem);
  const int na = axis == 1 ? ny : nz;
  const int n3 = axis == 1 ? nz : ny;
  const int nout = sub ? na / 2 : na;
  dim3 g((nx + kDpxCols - 1) / kDpxCols, need.out_n > 0 ? need.out_n : (nout + kDpxOut - 1) / kDpxOut,
         need.third_n > 0 ? need.third_n : (n3 + 1) / 2);
  // Full-resolution u16 tiles go through TMA (one box of the whole span per
  // third-axis slice) when the field's rows are whole 64-column boxes.
  // Measured at 1024^3: dilation z 2.71 -> 2.64 ms, centre erosion y
  // 1.27 -> 1.24 ms; the half-resolution lattice passes (sub) were a third
  // slower with TMA (0.63 -> 0.84, 0.31 -> 0.42 ms; 16-row boxes: slower
  // everywhere) and keep their per-thread loads.
  CUtensorMap tmap;
  memset(&tmap, 0, sizeof(tmap));
  int use_tma = 0;
  const int span = (sub ? 2 * kDpxOut - 1 : kDpxOut) + 2 * halo;
  if (sizeof(TIn) == 2 && sub == 0 && nx % kDpxCols == 0 && span <= 256 &&
      (reinterpret_cast<uintptr_t>(in) & 15) == 0)
    use_tma = encode_tensor_map_3d(&tmap, in, 2, nx, ny, nz, kDpxCols, axis == 1 ? span : 1, axis == 1 ? 1 : span)
                  ? 1
                  : 0;
  GM_LAUNCH(kc, name, st,
            k_pass_dpx<G, TIn, FIN><<<g, 256, smem, st>>>(in, out16, out8, nx, ny, nz, axis, sub, halo, cap, R,
                                                          uniform_r, rx, ry, rmap, rext, need, tmap, use_tma));
}

// ---- grouped min-plus passes (many grids, one persistent launch) ----
//
// One pass of the closing of many grids (the same pass of each: same
// kernel shape, own sizes, radius bounds, buffers and need maps), recorded
// by launch_close in phase mode and run as one launch: a grid of resident
// blocks pulls tiles of all the grids from one work counter, so that small
// grids fill the GPU together and the cost differences between tiles
// (window lengths vary with the local radius and the early exits) balance
// across blocks.  The tiles and their results are those of the per-grid
// launches (the same tile function on the same tile coordinates).
struct DpxJob {
  const void* in;
  uint16_t* out16;
  uint8_t* out8;
  int nx, ny, nz, axis, sub, halo;
  uint32_t cap;
  RField R;
  int uniform_r, rx, ry;
  const uint8_t* rmap;
  int rext;
  NeedMap need;
  int gx, gy, gz;  // tiles of this grid's pass
  int first;       // its first work item (tiles of the jobs before it)
};

// Instantiations a grouped launch may hold: the passes of launch_close.
enum DpxKind {
  DPXK_LAT_U8_0 = 0,   // sphere dilation y
  DPXK_LAT_U16_1,      // sphere dilation z (threshold + packing)
  DPXK_CUBE_U8_0,      // cube dilation y
  DPXK_CUBE_U16_1,     // cube dilation z
  DPXK_CEN2_U16_0,     // centre erosion y
  DPXK_CEN2_U16_2,     // centre erosion z
  DPXK_LAT2_U16_0,     // lattice-point erosion y
  DPXK_LAT2_U16_3,     // lattice-point erosion z
  DPXK_COUNT
};
template <int G, typename TIn, int FIN>
constexpr int dpx_kind() {
  return G == KERN_LAT && sizeof(TIn) == 1 && FIN == 0    ? DPXK_LAT_U8_0
         : G == KERN_LAT && sizeof(TIn) == 2 && FIN == 1  ? DPXK_LAT_U16_1
         : G == KERN_CUBE && sizeof(TIn) == 1 && FIN == 0 ? DPXK_CUBE_U8_0
         : G == KERN_CUBE && sizeof(TIn) == 2 && FIN == 1 ? DPXK_CUBE_U16_1
         : G == KERN_CEN2 && sizeof(TIn) == 2 && FIN == 0 ? DPXK_CEN2_U16_0
         : G == KERN_CEN2 && sizeof(TIn) == 2 && FIN == 2 ? DPXK_CEN2_U16_2
         : G == KERN_LAT2 && sizeof(TIn) == 2 && FIN == 0 ? DPXK_LAT2_U16_0
         : G == KERN_LAT2 && sizeof(TIn) == 2 && FIN == 3 ? DPXK_LAT2_U16_3
                                                          : -1;
}

template <int G, typename TIn, int FIN>
__global__ void __launch_bounds__(256, 4) k_pass_dpx_group(const DpxJob* __restrict__ jobs, int njobs, int total,
                                                        unsigned int* __restrict__ counter) {
  __shared__ int item_s;     // the block's current work item
  __shared__ int job_end_s;  // first item past the job held in job_s
  // the job of the current item (kept while the block's items stay in it)
  __shared__ __align__(16) unsigned char job_raw[sizeof(DpxJob)];
  DpxJob& job_s = *reinterpret_cast<DpxJob*>(job_raw);
  if (threadIdx.x == 0) {
    item_s = (int)atomicAdd(counter, 1u);
    job_end_s = -1;
  }
  __syncthreads();
  for (;;) {
    const int item = item_s;
    if (item >= total) return;  // block-uniform
    const bool other_job = item >= job_end_s || item < job_s.first;  // (job_end_s = -1 at first)
    // every thread has read job_s / job_end_s before warp 0 may rewrite
    // them, so that the branch below (and its barrier) is block-uniform
    __syncthreads();
    if (other_job) {
      if (threadIdx.x < 32) {
        // the job holding the item: the last one whose first item is <= it
        int lo = 0, hi = njobs - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (jobs[mid].first <= item) lo = mid; else hi = mid - 1;
        }
        const uint32_t* src = reinterpret_cast<const uint32_t*>(jobs + lo);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&job_s);
        for (int k = threadIdx.x; k < (int)(sizeof(DpxJob) / 4); k += 32) dst[k] = src[k];
        if (threadIdx.x == 0) job_end_s = jobs[lo].first + jobs[lo].gx * jobs[lo].gy * jobs[lo].gz;
      }
      __syncthreads();
    }
    // the next item, fetched while this tile runs (consumed after it)
    int next = 0;
    if (threadIdx.x == 0) next = (int)atomicAdd(counter, 1u);
    const DpxJob& b = job_s;
    const int t = item - b.first;
    const int bx = t % b.gx, by = (t / b.gx) % b.gy, bz = t / (b.gx * b.gy);
    dpx_tile<G, TIn, FIN>(static_cast<const TIn*>(b.in), b.out16, b.out8, b.nx, b.ny, b.nz, b.axis, b.sub, b.halo,
                          b.cap, b.R, b.uniform_r, b.rx, b.ry, b.rmap, b.rext, b.need, nullptr, 0,
                          bx, by + b.need.out0, bz + b.need.third0);
    __syncthreads();  // every thread is done with this tile (its shared memory, job_s, item_s)
    if (threadIdx.x == 0) item_s = next;
    __syncthreads();
  }
}

struct DpxGroup {
  int kind = -1;
  size_t smem = 0;
  std::vector<DpxJob> jobs;
  int total = 0;
  DpxJob* h_jobs = nullptr;  // pinned copy read by the upload (also at graph replays)
  DpxJob* d_jobs = nullptr;
  unsigned int* d_counter = nullptr;
  int cap = 0;
  cudaEvent_t uploaded = nullptr;  // after the last upload outside a capture (h_jobs free again)
};

DpxGroup* dpx_group_new() { return new DpxGroup(); }

void dpx_group_free(DpxGroup* g) {
  if (!g) return;
  if (g->uploaded) {
    cudaEventSynchronize(g->uploaded);
    cudaEventDestroy(g->uploaded);
  }
  if (g->h_jobs) cudaFreeHost(g->h_jobs);
  cudaFree(g->d_jobs);
  cudaFree(g->d_counter);
  delete g;
}

void dpx_group_clear(DpxGroup* g) {
  g->kind = -1;
  g->smem = 0;
  g->jobs.clear();
  g->total = 0;
}

int dpx_group_size(const DpxGroup* g) { return (int)g->jobs.size(); }

cudaError_t dpx_group_reserve(DpxGroup* g, int njobs) {
  if (njobs <= g->cap) return cudaSuccess;
  cudaError_t e;
  if (g->uploaded && (e = cudaEventSynchronize(g->uploaded)) != cudaSuccess) return e;
  if (!g->uploaded && (e = cudaEventCreateWithFlags(&g->uploaded, cudaEventDisableTiming)) != cudaSuccess) return e;
  if (g->h_jobs) cudaFreeHost(g->h_jobs);
  cudaFree(g->d_jobs);
  g->h_jobs = nullptr;
  g->d_jobs = nullptr;
  g->cap = 0;
  if ((e = cudaMallocHost(&g->h_jobs, sizeof(DpxJob) * njobs)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&g->d_jobs, sizeof(DpxJob) * njobs)) != cudaSuccess) return e;
  if (!g->d_counter && (e = cudaMalloc(&g->d_counter, sizeof(unsigned int))) != cudaSuccess) return e;
  g->cap = njobs;
  return cudaSuccess;
}

// Records one grid's pass (the arguments of launch_dpx) into the group.
template <int G, typename TIn, int FIN>
static bool dpx_record(DpxGroup* grp, const TIn* in, uint16_t* out16, uint8_t* out8, int nx, int ny, int nz, int axis,
                       int sub, int halo, uint32_t cap, RField R, int uniform_r, int rx, int ry,
                       const uint8_t* rmap, int rext, NeedMap need) {
  constexpr int kind = dpx_kind<G, TIn, FIN>();
  if (kind < 0 || (grp->kind >= 0 && grp->kind != kind) || (G == KERN_LAT2) != (sub != 0)) return false;
  grp->kind = kind;
  grp->smem = std::max(grp->smem, dpx_smem_bytes(sub, halo));
  const int na = axis == 1 ? ny : nz;
  const int n3 = axis == 1 ? nz : ny;
  const int nout = sub ? na / 2 : na;
  DpxJob j;
  j.in = in;
  j.out16 = out16;
  j.out8 = out8;
  j.nx = nx;
  j.ny = ny;
  j.nz = nz;
  j.axis = axis;
  j.sub = sub;
  j.halo = halo;
  j.cap = cap;
  j.R = R;
  j.uniform_r = uniform_r;
  j.rx = rx;
  j.ry = ry;
  j.rmap = rmap;
  j.rext = rext;
  j.need = need;
  j.gx = (nx + kDpxCols - 1) / kDpxCols;
  j.gy = need.out_n > 0 ? need.out_n : (nout + kDpxOut - 1) / kDpxOut;
  j.gz = need.third_n > 0 ? need.third_n : (n3 + 1) / 2;
  j.first = grp->total;
  const long long tiles = (long long)j.gx * j.gy * j.gz;
  if (tiles <= 0) return true;
  if (grp->total + tiles > 0x7fffffffLL) return false;
  grp->total += (int)tiles;
  grp->jobs.push_back(j);
  return true;
}

static const char* const kDpxGroupNames[DPXK_COUNT] = {
    "k_pass_dil_y_group", "k_pass_dil_z_group",  "k_pass_dil_y_group",  "k_pass_dil_z_group",
    "k_pass_ero_y_group", "k_pass_ero_z_group", "k_pass_erob_y_group", "k_pass_erob_z_group"};

template <int G, typename TIn, int FIN>
static cudaError_t dpx_group_go(DpxGroup* g, int sms, cudaStream_t st, KernelCounter* kc) {
  const void* k = reinterpret_cast<const void*>(k_pass_dpx_group<G, TIn, FIN>);
  cudaError_t e = ensure_dynamic_smem(k, g->smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pass_dpx_group<G, TIn, FIN>, 256, g->smem)) !=
      cudaSuccess)
    return e;
  const int blocks = std::max(1, std::min(g->total, std::max(1, sms) * std::max(1, per_sm)));
  GM_LAUNCH(kc, kDpxGroupNames[g->kind], st,
            k_pass_dpx_group<G, TIn, FIN><<<blocks, 256, g->smem, st>>>(g->d_jobs, (int)g->jobs.size(), g->total,
                                                                        g->d_counter));
  return cudaGetLastError();
}

cudaError_t dpx_group_launch(DpxGroup* g, int sms, cudaStream_t st, KernelCounter* kc) {
  if (g->jobs.empty()) return cudaSuccess;
  const int n = (int)g->jobs.size();
  if (n > g->cap) return cudaErrorInvalidValue;  // dpx_group_reserve first (not while capturing)
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cs);
  if (e != cudaSuccess) return e;
  const bool capturing = cs == cudaStreamCaptureStatusActive;
  // the previous upload has read the pinned table (in a capture the caller
  // guarantees that no replay of an earlier graph over it is in flight)
  if (!capturing && (e = cudaEventSynchronize(g->uploaded)) != cudaSuccess) return e;
  memcpy(g->h_jobs, g->jobs.data(), sizeof(DpxJob) * n);
  if ((e = cudaMemcpyAsync(g->d_jobs, g->h_jobs, sizeof(DpxJob) * n, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  if (!capturing && (e = cudaEventRecord(g->uploaded, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(g->d_counter, 0, sizeof(unsigned int), st)) != cudaSuccess) return e;
  switch (g->kind) {
    case DPXK_LAT_U8_0: return dpx_group_go<KERN_LAT, uint8_t, 0>(g, sms, st, kc);
    case DPXK_LAT_U16_1: return dpx_group_go<KERN_LAT, uint16_t, 1>(g, sms, st, kc);
    case DPXK_CUBE_U8_0: return dpx_group_go<KERN_CUBE, uint8_t, 0>(g, sms, st, kc);
    case DPXK_CUBE_U16_1: return dpx_group_go<KERN_CUBE, uint16_t, 1>(g, sms, st, kc);
    case DPXK_CEN2_U16_0: return dpx_group_go<KERN_CEN2, uint16_t, 0>(g, sms, st, kc);
    case DPXK_CEN2_U16_2: return dpx_group_go<KERN_CEN2, uint16_t, 2>(g, sms, st, kc);
    case DPXK_LAT2_U16_0: return dpx_group_go<KERN_LAT2, uint16_t, 0>(g, sms, st, kc);
    case DPXK_LAT2_U16_3: return dpx_group_go<KERN_LAT2, uint16_t, 3>(g, sms, st, kc);
    default: return cudaErrorInvalidValue;
  }
}

// A pass of launch_close: launched (a.phase < 0), recorded into a.group
// when it is the pass of the phase asked for, or skipped.  `at` counts the
// passes met so far.
template <int G, typename TIn, int FIN>
static bool dpx_step(const CloseArgs& a, int& at, const TIn* in, uint16_t* out16, uint8_t* out8, int nx, int ny,
                     int nz, int axis, int sub, int halo, uint32_t cap, RField R, int uniform_r, int rx, int ry,
                     cudaStream_t st, KernelCounter* kc, const char* name, const uint8_t* rmap = nullptr,
                     int rext = 0,
                     NeedMap need = NeedMap{nullptr, 0, 0, 0, 0, 0, 0, 0, 0,
                                            CBox{{0, 0, 0}, {1 << 30, 1 << 30, 1 << 30}}}) {
  bool ok = true;
  if (a.phase < 0)
    launch_dpx<G, TIn, FIN>(in, out16, out8, nx, ny, nz, axis, sub, halo, cap, R, uniform_r, rx, ry, st, kc, name,
                            rmap, rext, need);
  else if (a.phase == at)
    ok = a.group != nullptr && dpx_record<G, TIn, FIN>(a.group, in, out16, out8, nx, ny, nz, axis, sub, halo, cap, R,
                                                        uniform_r, rx, ry, rmap, rext, need);
  at++;
  return ok;
}

// The driver's tensor-map encoder, looked up once per process (before any
// stream capture: gm_ctx_create calls tma_init).
static PFN_cuTensorMapEncodeTiled_v12000 tma_encoder() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    cudaGetLastError();
  });
  return encode;
}

void tma_init() { tma_encoder(); }

bool encode_tensor_map_3d(CUtensorMap* map, const void* base, int elem_bytes, int nx, int ny, int nz, int bx, int by,
                          int bz) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tma_encoder();
  if (encode == nullptr || (elem_bytes != 1 && elem_bytes != 2)) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)nx * elem_bytes, (cuuint64_t)nx * ny * elem_bytes};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode(map, elem_bytes == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 3,
                const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t kernel_error_flags(unsigned int* flags, bool clear) {
  cudaError_t e = cudaMemcpyFromSymbol(flags, g_kernel_errors, sizeof(unsigned int));
  if (e == cudaSuccess && clear && *flags != 0) {
    const unsigned int zero = 0;
    e = cudaMemcpyToSymbol(g_kernel_errors, &zero, sizeof(unsigned int));
  }
  return e;
}

// Largest raw radius (>= 0) of each 16^3 block of fine voxels of a radius
// field (nx, ny, nz multiples of 16, nx <= 16 * 32 * kRmapCells).  One block
// per (map y, map z) row of map cells; a warp reads whole fine rows (lane l
// owns the 16-byte segments of map cells l, l + 32, ...), the 8 warps take
// every 8th of the 256 rows, so the block streams its 16 x 16 rows of the
// field front to back.  With d_rmax, the largest clamped radius is folded
// into *d_rmax as well.
constexpr int kRmapCells = 4;  // map cells per lane along x
__global__ void __launch_bounds__(256) k_radius_map(RField R, int mbx, int mby, int aligned,
                                                     uint8_t* __restrict__ out, int* __restrict__ d_rmax) {
  const int my = blockIdx.x, mz = blockIdx.y;
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ int part[8][32 * kRmapCells];
  int m[kRmapCells];
#pragma unroll
  for (int c = 0; c < kRmapCells; c++) m[c] = 0;
  if (aligned) {
    uint32_t m4[kRmapCells];
#pragma unroll
    for (int c = 0; c < kRmapCells; c++) m4[c] = 0u;
#pragma unroll 2
    for (int r = wid; r < 256; r += 8) {
      const int8_t* row = R.p + (int64_t)(16 * my + (r & 15)) * R.sy + (int64_t)(16 * mz + (r >> 4)) * R.sz;
#pragma unroll
      for (int c = 0; c < kRmapCells; c++) {
        const int cx = lane + 32 * c;
        if (cx < mbx) {
          const uint4 v = __ldcs(reinterpret_cast<const uint4*>(row + 16 * cx));
          m4[c] = __vmaxs4(m4[c], __vmaxs4(__vmaxs4(v.x, v.y), __vmaxs4(v.z, v.w)));  // per-byte signed maxima
        }
      }
    }
#pragma unroll
    for (int c = 0; c < kRmapCells; c++)
#pragma unroll
      for (int j = 0; j < 4; j++) m[c] = max(m[c], (int)((m4[c] >> (8 * j)) & 0xffu));  // bytes >= 0 here
  } else {
    for (int r = wid; r < 256; r += 8) {
      const int8_t* row = R.p + (int64_t)(16 * my + (r & 15)) * R.sy + (int64_t)(16 * mz + (r >> 4)) * R.sz;
#pragma unroll
      for (int c = 0; c < kRmapCells; c++) {
        const int cx = lane + 32 * c;
        if (cx < mbx)
#pragma unroll
          for (int j = 0; j < 16; j++) m[c] = max(m[c], (int)row[16 * cx + j]);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < kRmapCells; c++) part[wid][lane + 32 * c] = m[c];
  __syncthreads();
  int gmax = 0;
  for (int cx = threadIdx.x; cx < mbx; cx += blockDim.x) {
    int t = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) t = max(t, part[k][cx]);
    out[cx + (int64_t)mbx * (my + (int64_t)mby * mz)] = (uint8_t)t;
    gmax = max(gmax, t);
  }
  if (d_rmax != nullptr && wid * 32 < mbx) {
    for (int o = 16; o > 0; o >>= 1) gmax = max(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
    if (lane == 0) atomicMax(d_rmax, clamp_radius(gmax));
  }
}

cudaError_t launch_radius_map(RField R, int nx, int ny, int nz, uint8_t* out, int* d_rmax, cudaStream_t st,
                              KernelCounter* kc) {
  const int mbx = nx / 16, mby = ny / 16, mbz = nz / 16;
  if (mbx > 32 * kRmapCells) return cudaErrorInvalidValue;
  const int aligned = ((uintptr_t)R.p % 16 == 0 && R.sy % 16 == 0 && R.sz % 16 == 0) ? 1 : 0;
  if (d_rmax) cudaMemsetAsync(d_rmax, 0, sizeof(int), st);
  GM_LAUNCH(kc, "k_radius_map", st, k_radius_map<<<dim3(mby, mbz), 256, 0, st>>>(R, mbx, mby, aligned, out, d_rmax));
  return cudaGetLastError();
}

cudaError_t launch_radius_map_dense(const int8_t* R, int nx, int ny, int nz, uint8_t* out, int* d_rmax,
                                    cudaStream_t st, KernelCounter* kc) {
  return launch_radius_map(RField{R, (int64_t)nx, (int64_t)nx * ny}, nx, ny, nz, out, d_rmax, st, kc);
}

// 1 for each 8^3 block of cells of a cell grid (rx, ry, rz multiples of
// 16) holding a non-zero byte: one warp per block, two 8-byte rows a lane.
__global__ void __launch_bounds__(256) k_occ_map8(const uint8_t* __restrict__ G, int rx, int ry, int mdx, int mdy,
                                                  int nblocks, uint8_t* __restrict__ out) {
  const int b = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (b >= nblocks) return;
  const int bx = b % mdx, by = (b / mdx) % mdy, bz = b / (mdx * mdy);
  uint64_t acc = 0;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int r = lane + 32 * k;  // row r of the block: y = r & 7, z = r >> 3
    acc |= *reinterpret_cast<const uint64_t*>(G + idx3(8 * bx, 8 * by + (r & 7), 8 * bz + (r >> 3), rx, ry));
  }
  const int any = __any_sync(0xffffffffu, acc != 0);
  if (lane == 0) out[b] = any ? 1 : 0;
}

// ---------------------------------------------------------------------
// cell-level kernels
// ---------------------------------------------------------------------

struct DataRes { int v[3]; };

// ---------------------------------------------------------------------
// cell-level kernels; cell grids of this section are boxes of rx * ry * rz
// cells (Dims), z = blockIdx.z
// ---------------------------------------------------------------------

struct Dims { int x, y, z; };
__device__ __forceinline__ int64_t cidx(int x, int y, int z, Dims d) { return idx3(x, y, z, d.x, d.y); }

// Dilation flags from a resident squared lattice distance field E of the
// input grid (u16 per fine voxel: the value the dilation's z pass computes,
// saturated at (rmax + 1)^2 for a bound rmax of every radius asked for).
// The flag of fine voxel p is E(p) < (r(p) + 1)^2, the z pass's own test, so
// the bytes equal the passes' output.  Four cells per thread, bit
// x + 2y + 4z of the 2x2x2 fine voxels of a cell.
__global__ void __launch_bounds__(256) k_dil_threshold(const uint16_t* __restrict__ E, int64_t esy, int64_t esz,
                                                       RField R, int uniform_r, Dims g, uint8_t* __restrict__ out,
                                                       CBox roi) {
  const int x4 = 4 * (blockIdx.x * 64 + threadIdx.x);
  const int y = blockIdx.y * 4 + threadIdx.y, z = blockIdx.z;
  if (x4 >= g.x || y >= g.y || !cbox_meets(roi, x4, x4 + 3, y, y, z, z)) return;
  const int ru = clamp_radius(uniform_r);
  uint32_t out4 = 0;
#pragma unroll
  for (int r = 0; r < 4; r++) {  // fine row: y parity r & 1, z parity r >> 1
    const int fy = 2 * y + (r & 1), fz = 2 * z + (r >> 1);
    const uint16_t* er = E + fy * esy + fz * esz + 2 * x4;
    const int8_t* rr = R.p != nullptr ? R.p + fy * R.sy + fz * R.sz + 2 * x4 : nullptr;
#pragma unroll
    for (int i = 0; i < 4; i++) {  // fine x 2(x4 + i) and 2(x4 + i) + 1
      const uint32_t e2 = *reinterpret_cast<const uint32_t*>(er + 2 * i);
      int r0 = ru, r1 = ru;
      if (rr != nullptr) {
        const uint32_t w = *reinterpret_cast<const uint16_t*>(rr + 2 * i);
        r0 = clamp_radius((int)(int8_t)(w & 0xffu));
        r1 = clamp_radius((int)(int8_t)(w >> 8));
      }
      const uint32_t b0 = (e2 & 0xffffu) < (uint32_t)((r0 + 1) * (r0 + 1)) ? 1u : 0u;
      const uint32_t b1 = (e2 >> 16) < (uint32_t)((r1 + 1) * (r1 + 1)) ? 2u : 0u;
      out4 |= (b0 | b1) << (2 * r + 8 * i);
    }
  }
  *reinterpret_cast<uint32_t*>(out + cidx(x4, y, z, g)) = out4;
}


__device__ __forceinline__ uint32_t c0_of(uint32_t x, uint32_t d, uint32_t eb, bool inside) {
  return (inside && d != 0u && x != 0xffu && eb) ? 0u : d;
}


static dim3 quad_grid(Dims g) { return dim3((g.x / 4 + 63) / 64, (g.y + 3) / 4, g.z); }

// ---------------------------------------------------------------------
// The same cell-level kernels on 16 consecutive cells per thread (one
// 16-byte load per row), four cells per 32-bit word at a time: the
// per-byte rules become byte masks (__vcmp*4) and shifts that stay within
// bytes.  Block (32, 8): x along threadIdx.x, y along threadIdx.y.
// ---------------------------------------------------------------------

__device__ __forceinline__ uint4 ld16(const uint8_t* g, int x16, int y, int z, Dims d) {
  return *reinterpret_cast<const uint4*>(g + cidx(x16, y, z, d));
}
__device__ __forceinline__ uint32_t w_of(const uint4& q, int j) {
  return j == 0 ? q.x : (j == 1 ? q.y : (j == 2 ? q.z : q.w));
}
// 0xff in byte i where cell x0 + i satisfies lo <= x < hi
__device__ __forceinline__ uint32_t xrange_mask(int x0, int lo, int hi) {
  uint32_t m = 0;
#pragma unroll
  for (int i = 0; i < 4; i++) m |= (x0 + i >= lo && x0 + i < hi) ? (0xffu << (8 * i)) : 0u;
  return m;
}
// the word of cells x0 + 1 .. x0 + 4 (x0 - 1 .. x0 + 2) from the word of
// x0 .. x0 + 3 and the byte after (before) it
__device__ __forceinline__ uint32_t next_cells(uint32_t w, uint32_t after) { return (w >> 8) | (after << 24); }
__device__ __forceinline__ uint32_t prev_cells(uint32_t w, uint32_t before) { return (w << 8) | before; }

// Contour of the dilation: fine voxels outside D that are 6-adjacent to D.
// GM_REF: only for cells in [1, res-2]^3 whose byte is not 0xff
// (TagVoxelsContourByErosion, Grid.cu:1230-1327); GM_EXACT: whole grid.
// A block of 32 x 10 threads walks kConZ cells along z, each thread
// keeping its row of D at z - 1, z, z + 1 in registers; the rows y - 1 and
// y + 1 come from the neighbouring warps through shared memory (warps 0 and
// 9 load the halo rows only) and the bytes before and after a thread's 16
// cells from its neighbouring lanes, so each row of D is read once.
constexpr int kConZ = 16;
__global__ void __launch_bounds__(320) k_contour_z(const uint8_t* __restrict__ D, uint8_t* __restrict__ S, Dims g,
                                                   int exact, CBox roi) {
  __shared__ uint4 rows_s[10][32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x16 = 16 * (blockIdx.x * 32 + tx);
  const int y = (int)blockIdx.y * 8 - 1 + ty;
  const int z0 = (int)blockIdx.z * kConZ, z1 = min(z0 + kConZ, g.z);
  const bool xok = x16 < g.x, yok = y >= 0 && y < g.y;
  const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
  auto row = [&](int zz) { return xok && yok && zz >= 0 && zz < g.z ? ld16(D, x16, y, zz, g) : z4; };
  uint4 zm = row(z0 - 1), v = row(z0);
  for (int z = z0; z < z1; z++) {
    const uint4 zp = row(z + 1);
    rows_s[ty][tx] = v;
    __syncthreads();
    uint32_t before = __shfl_up_sync(0xffffffffu, v.w >> 24, 1);
    uint32_t after = __shfl_down_sync(0xffffffffu, v.x & 0xffu, 1);
    if (ty >= 1 && ty <= 8 && xok && yok && cbox_meets(roi, x16, x16 + 15, y, y, z, z)) {
      if (tx == 0) before = x16 > 0 ? D[cidx(x16 - 1, y, z, g)] : 0u;
      if (tx == 31 || x16 + 16 >= g.x) after = x16 + 16 < g.x ? D[cidx(x16 + 16, y, z, g)] : 0u;
      const uint4 ym = rows_s[ty - 1][tx], yp = rows_s[ty + 1][tx];
      const bool yz_in = y >= 1 && z >= 1 && y <= g.y - 2 && z <= g.z - 2;
      uint32_t o[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const uint32_t vw = w_of(v, j);
        const uint32_t l = prev_cells(vw, j > 0 ? w_of(v, j - 1) >> 24 : before);
        const uint32_t r = next_cells(vw, j < 3 ? w_of(v, j + 1) & 0xffu : after);
        // 6-neighbours of each fine voxel (bit x + 2y + 4z of a byte)
        uint32_t t = ((vw & 0xAAAAAAAAu) >> 1) | ((r & 0x55555555u) << 1);
        t |= ((vw & 0x55555555u) << 1) | ((l & 0xAAAAAAAAu) >> 1);
        t |= ((vw & 0xCCCCCCCCu) >> 2) | ((w_of(yp, j) & 0x33333333u) << 2);
        t |= ((vw & 0x33333333u) << 2) | ((w_of(ym, j) & 0xCCCCCCCCu) >> 2);
        t |= ((vw & 0xF0F0F0F0u) >> 4) | ((w_of(zp, j) & 0x0F0F0F0Fu) << 4);
        t |= ((vw & 0x0F0F0F0Fu) << 4) | ((w_of(zm, j) & 0xF0F0F0F0u) >> 4);
        uint32_t m = 0xffffffffu;
        if (!exact) m = yz_in ? (__vcmpne4(vw, 0xffffffffu) & xrange_mask(x16 + 4 * j, 1, g.x - 1)) : 0u;
        o[j] = t & ~vw & m;
      }
      *reinterpret_cast<uint4*>(S + cidx(x16, y, z, g)) = make_uint4(o[0], o[1], o[2], o[3]);
    }
    __syncthreads();  // rows_s is rewritten for the next z
    zm = v;
    v = zp;
  }
}

// GM_REF dilation select: base pass (cells inside data_res that are not
// full take 0xff when their child-0 corner is dilated, GMorpho.cu:2848-2927)
// then the tight contour (forward 2x2x2 block mixes full and non-full,
// Grid.cu:1589-1607) takes the fine per-voxel byte (GMorpho.cu:2930-3056).
//
// base-pass bytes of the dilation (GM_REF) of one row of 16 cells and the
// full flags (0xff per full byte) of the cells x16 + 1 .. x16 + 16
__device__ __forceinline__ void base_dil_row(const uint8_t* X, const uint8_t* Df, int x16, int yy, int zz, Dims g,
                                             const DataRes& dr, uint32_t d0[4], uint32_t f[4], uint32_t fr[4],
                                             uint32_t dfw[4]) {
  if (yy >= g.y || zz >= g.z) {
#pragma unroll
    for (int j = 0; j < 4; j++) { d0[j] = 0u; f[j] = 0u; fr[j] = 0u; dfw[j] = 0u; }
    return;
  }
  const bool iyz = yy < dr.v[1] && zz < dr.v[2];
  const uint4 xq = ld16(X, x16, yy, zz, g), dq = ld16(Df, x16, yy, zz, g);
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const uint32_t xw = w_of(xq, j), dw = w_of(dq, j);
    const uint32_t in = iyz ? xrange_mask(x16 + 4 * j, 0, dr.v[0]) : 0u;
    const uint32_t cond = in & __vcmpne4(xw, 0xffffffffu) & ((dw & 0x01010101u) * 0xffu);
    d0[j] = xw | cond;
    f[j] = __vcmpeq4(d0[j], 0xffffffffu);
    dfw[j] = dw;
  }
  // full flag of cell x16 + 16
  uint32_t fa = 0u;
  if (x16 + 16 < g.x) {
    const int64_t c = cidx(x16 + 16, yy, zz, g);
    const uint32_t xb = X[c], db = Df[c];
    const bool inside = iyz && x16 + 16 < dr.v[0];
    const uint32_t d = (inside && xb != 0xffu && (db & 1u)) ? 0xffu : xb;
    fa = d == 0xffu ? 0xffu : 0u;
  }
#pragma unroll
  for (int j = 0; j < 4; j++) fr[j] = next_cells(f[j], j < 3 ? f[j + 1] & 0xffu : fa);
}

// The select kernel computes each base-pass row once: a block of 32 x 9
// threads walks kSelZ cells along z, each thread keeping its row's flags at
// z and z + 1 in registers; the row y + 1 comes from the next warp through
// shared memory (warp 8 computes that halo row only).
constexpr int kSelZ = 16;
__global__ void __launch_bounds__(288) k_dil_select_z(const uint8_t* __restrict__ X, const uint8_t* __restrict__ Df,
                                                      uint8_t* __restrict__ D, Dims g, DataRes dr, CBox roi) {
  __shared__ uint4 flags_s[9][32][4];  // per thread: f, fr at z; f, fr at z + 1
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x16 = 16 * (blockIdx.x * 32 + tx);
  const int y = (int)blockIdx.y * 8 + ty;
  const int z0 = (int)blockIdx.z * kSelZ, z1 = min(z0 + kSelZ, g.z);
  const bool xok = x16 < g.x;
  auto row = [&](int zz, uint32_t d0[4], uint32_t f[4], uint32_t fr[4], uint32_t dfw[4]) {
    if (xok) {
      base_dil_row(X, Df, x16, y, zz, g, dr, d0, f, fr, dfw);  // zeros outside the grid
    } else {
#pragma unroll
      for (int j = 0; j < 4; j++) d0[j] = f[j] = fr[j] = dfw[j] = 0u;
    }
  };
  uint32_t d0c[4], fc[4], frc[4], dfc[4];
  row(z0, d0c, fc, frc, dfc);
  for (int z = z0; z < z1; z++) {
    uint32_t d0n[4], fn[4], frn[4], dfn[4];
    row(z + 1, d0n, fn, frn, dfn);
    flags_s[ty][tx][0] = make_uint4(fc[0], fc[1], fc[2], fc[3]);
    flags_s[ty][tx][1] = make_uint4(frc[0], frc[1], frc[2], frc[3]);
    flags_s[ty][tx][2] = make_uint4(fn[0], fn[1], fn[2], fn[3]);
    flags_s[ty][tx][3] = make_uint4(frn[0], frn[1], frn[2], frn[3]);
    __syncthreads();
    if (ty < 8 && xok && y < g.y && cbox_meets(roi, x16, x16 + 15, y, y, z, z)) {
      const uint4 f1 = flags_s[ty + 1][tx][0], fr1 = flags_s[ty + 1][tx][1];
      const uint4 f2 = flags_s[ty + 1][tx][2], fr2 = flags_s[ty + 1][tx][3];
      // the forward 2x2x2 block mixes full and non-full bytes (cells <= dims - 2)
      const bool yz_ok = y <= g.y - 2 && z <= g.z - 2;
      uint32_t o[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const uint32_t any = fc[j] | frc[j] | fn[j] | frn[j] | w_of(f1, j) | w_of(fr1, j) | w_of(f2, j) | w_of(fr2, j);
        const uint32_t all = fc[j] & frc[j] & fn[j] & frn[j] & w_of(f1, j) & w_of(fr1, j) & w_of(f2, j) & w_of(fr2, j);
        const uint32_t tag = yz_ok ? (any & ~all & xrange_mask(x16 + 4 * j, 0, g.x - 1)) : 0u;
        o[j] = (tag & dfc[j]) | (~tag & d0c[j]);
      }
      *reinterpret_cast<uint4*>(D + cidx(x16, y, z, g)) = make_uint4(o[0], o[1], o[2], o[3]);
    }
    __syncthreads();  // flags_s is rewritten for the next z
#pragma unroll
    for (int j = 0; j < 4; j++) {
      d0c[j] = d0n[j];
      fc[j] = fn[j];
      frc[j] = frn[j];
      dfc[j] = dfn[j];
    }
  }
}

// GM_REF erosion select: base pass (cells inside data_res with D != 0 and
// X != 0xff are cleared when the centre 2c+1 is eroded, GMorpho.cu:4360-4370,
// 4644-4646), then cells whose byte differs from a 6-neighbour
// (Grid.cu:1499-1570) take 0xff & ~eroded (GMorpho.cu:5353-5360).
//
// C0 = base erosion of 16 cells of one row: 0 where the cell is inside the
// data, D != 0, X != 0xff and its lattice point 2c+1 is eroded; D otherwise
__device__ __forceinline__ void base_ero_row(const uint8_t* X, const uint8_t* D, const uint8_t* Eb, int x16, int yy,
                                             int zz, Dims g, const DataRes& dr, uint32_t c0[4]) {
  const bool iyz = yy < dr.v[1] && zz < dr.v[2];
  const uint4 xq = ld16(X, x16, yy, zz, g), dq = ld16(D, x16, yy, zz, g), eq = ld16(Eb, x16, yy, zz, g);
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const uint32_t dw = w_of(dq, j);
    const uint32_t in = iyz ? xrange_mask(x16 + 4 * j, 0, dr.v[0]) : 0u;
    const uint32_t cond = in & __vcmpne4(dw, 0u) & __vcmpne4(w_of(xq, j), 0xffffffffu) & __vcmpne4(w_of(eq, j), 0u);
    c0[j] = dw & ~cond;
  }
}

__global__ void __launch_bounds__(256) k_ero_select16(const uint8_t* __restrict__ X, const uint8_t* __restrict__ D,
                                                      const uint8_t* __restrict__ Eb, const uint8_t* __restrict__ Ef,
                                                      uint8_t* __restrict__ C, Dims g, DataRes dr, int exact,
                                                      CBox roi) {
  const int x16 = 16 * (blockIdx.x * 32 + threadIdx.x);
  const int y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
  if (x16 >= g.x || y >= g.y || !cbox_meets(roi, x16, x16 + 15, y, y, z, z)) return;
  const uint4 ef = ld16(Ef, x16, y, z, g);
  if (exact) {
    const uint4 d = ld16(D, x16, y, z, g);
    *reinterpret_cast<uint4*>(C + cidx(x16, y, z, g)) =
        make_uint4(d.x & ~ef.x, d.y & ~ef.y, d.z & ~ef.z, d.w & ~ef.w);
    return;
  }
  uint32_t c0[4];
  base_ero_row(X, D, Eb, x16, y, z, g, dr, c0);
  // C0 of the cells x16 - 1 and x16 + 16
  const bool iyz = y < dr.v[1] && z < dr.v[2];
  uint32_t before = 0u, after = 0u;
  if (x16 > 0) {
    const int64_t c = cidx(x16 - 1, y, z, g);
    before = c0_of(X[c], D[c], Eb[c], iyz && x16 - 1 < dr.v[0]);
  }
  if (x16 + 16 < g.x) {
    const int64_t c = cidx(x16 + 16, y, z, g);
    after = c0_of(X[c], D[c], Eb[c], iyz && x16 + 16 < dr.v[0]);
  }
  const bool interior_yz = y >= 1 && z >= 1 && y <= g.y - 2 && z <= g.z - 2;
  uint32_t diff[4] = {0u, 0u, 0u, 0u};
  if (interior_yz) {
    const int ny[4] = {y - 1, y + 1, y, y};
    const int nz[4] = {z, z, z - 1, z + 1};
#pragma unroll
    for (int n = 0; n < 4; n++) {
      uint32_t cn[4];
      base_ero_row(X, D, Eb, x16, ny[n], nz[n], g, dr, cn);
#pragma unroll
      for (int j = 0; j < 4; j++) diff[j] |= __vcmpne4(c0[j], cn[j]);
    }
  }
  uint32_t o[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const uint32_t l = prev_cells(c0[j], j > 0 ? c0[j - 1] >> 24 : before);
    const uint32_t r = next_cells(c0[j], j < 3 ? c0[j + 1] & 0xffu : after);
    const uint32_t tag = interior_yz ? ((diff[j] | __vcmpne4(c0[j], l) | __vcmpne4(c0[j], r)) &
                                        xrange_mask(x16 + 4 * j, 1, g.x - 1))
                                     : 0u;
    o[j] = (tag & ~w_of(ef, j)) | (~tag & c0[j]);
  }
  *reinterpret_cast<uint4*>(C + cidx(x16, y, z, g)) = make_uint4(o[0], o[1], o[2], o[3]);
}

static dim3 grid16(Dims g) { return dim3((g.x / 16 + 31) / 32, (g.y + 7) / 8, g.z); }

// GM_REF erosion select in two steps, so that the centre erosion Ef is
// computed only where it is read.  k_ero_tag_z writes the base erosion C0
// into C (final for untagged cells), the refinement tags (0xff per tagged
// cell) into T and marks the 8^3-cell blocks holding a tagged cell in tmap
// (zeroed by the caller); once Ef is known on those blocks, k_ero_fix16
// writes 0xff & ~Ef on the tagged cells.  The bytes equal k_ero_select16's.
// The tag kernel computes each base-erosion row once: a block of 32 x 10
// threads walks kTagZ cells along z, each thread keeping its row's C0 at
// z - 1, z, z + 1 in registers; the rows y - 1 and y + 1 at z come from
// the neighbouring warps through shared memory (warps 0 and 9 compute the
// halo rows only), and the bytes before and after a thread's 16 cells from
// its neighbouring lanes.
constexpr int kTagZ = 16;
__global__ void __launch_bounds__(320) k_ero_tag_z(const uint8_t* __restrict__ X, const uint8_t* __restrict__ D,
                                                   const uint8_t* __restrict__ Eb, uint8_t* __restrict__ C,
                                                   uint8_t* __restrict__ T, uint8_t* __restrict__ tmap, int mdx,
                                                   int mdy, Dims g, DataRes dr, CBox roi) {
  __shared__ uint4 rows_s[10][32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x16 = 16 * (blockIdx.x * 32 + tx);
  const int y = (int)blockIdx.y * 8 - 1 + ty;
  const int z0 = (int)blockIdx.z * kTagZ, z1 = min(z0 + kTagZ, g.z);
  const bool xok = x16 < g.x, yok = y >= 0 && y < g.y;
  auto row = [&](int zz, uint32_t c[4]) {
    if (xok && yok && zz >= 0 && zz < g.z) {
      base_ero_row(X, D, Eb, x16, y, zz, g, dr, c);
    } else {
#pragma unroll
      for (int j = 0; j < 4; j++) c[j] = 0u;
    }
  };
  uint32_t cp[4], cc[4], cn[4];
  row(z0 - 1, cp);
  row(z0, cc);
  for (int z = z0; z < z1; z++) {
    row(z + 1, cn);
    rows_s[ty][tx] = make_uint4(cc[0], cc[1], cc[2], cc[3]);
    __syncthreads();
    // C0 of the cells x16 - 1 and x16 + 16 (the neighbouring lanes' rows;
    // at the block's x edges, from the grid)
    uint32_t before = __shfl_up_sync(0xffffffffu, cc[3] >> 24, 1);
    uint32_t after = __shfl_down_sync(0xffffffffu, cc[0] & 0xffu, 1);
    const bool out = ty >= 1 && ty <= 8 && xok && yok && cbox_meets(roi, x16, x16 + 15, y, y, z, z);
    if (out) {
      const bool iyz = y < dr.v[1] && z < dr.v[2];
      if (tx == 0)
        before = 0u;
      if (tx == 0 && x16 > 0) {
        const int64_t c = cidx(x16 - 1, y, z, g);
        before = c0_of(X[c], D[c], Eb[c], iyz && x16 - 1 < dr.v[0]);
      }
      if (tx == 31 || x16 + 16 >= g.x) after = 0u;
      if (tx == 31 && x16 + 16 < g.x) {
        const int64_t c = cidx(x16 + 16, y, z, g);
        after = c0_of(X[c], D[c], Eb[c], iyz && x16 + 16 < dr.v[0]);
      }
      const bool interior_yz = y >= 1 && z >= 1 && y <= g.y - 2 && z <= g.z - 2;
      uint32_t tag[4] = {0u, 0u, 0u, 0u};
      if (interior_yz) {
        const uint4 ym = rows_s[ty - 1][tx], yp = rows_s[ty + 1][tx];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const uint32_t diff = __vcmpne4(cc[j], w_of(ym, j)) | __vcmpne4(cc[j], w_of(yp, j)) |
                                __vcmpne4(cc[j], cp[j]) | __vcmpne4(cc[j], cn[j]);
          const uint32_t l = prev_cells(cc[j], j > 0 ? cc[j - 1] >> 24 : before);
          const uint32_t r = next_cells(cc[j], j < 3 ? cc[j + 1] & 0xffu : after);
          tag[j] = (diff | __vcmpne4(cc[j], l) | __vcmpne4(cc[j], r)) & xrange_mask(x16 + 4 * j, 1, g.x - 1);
        }
      }
      const int64_t o = cidx(x16, y, z, g);
      *reinterpret_cast<uint4*>(C + o) = make_uint4(cc[0], cc[1], cc[2], cc[3]);
      *reinterpret_cast<uint4*>(T + o) = make_uint4(tag[0], tag[1], tag[2], tag[3]);
      const int64_t mb = idx3(x16 >> 3, y >> 3, z >> 3, mdx, mdy);
      if (tag[0] | tag[1]) tmap[mb] = 1;
      if (tag[2] | tag[3]) tmap[mb + 1] = 1;
    }
    __syncthreads();  // rows_s is rewritten for the next z
#pragma unroll
    for (int j = 0; j < 4; j++) {
      cp[j] = cc[j];
      cc[j] = cn[j];
    }
  }
}

__global__ void __launch_bounds__(256) k_ero_fix16(const uint8_t* __restrict__ T, const uint8_t* __restrict__ Ef,
                                                   uint8_t* __restrict__ C, Dims g, CBox roi) {
  const int x16 = 16 * (blockIdx.x * 32 + threadIdx.x);
  const int y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
  if (x16 >= g.x || y >= g.y || !cbox_meets(roi, x16, x16 + 15, y, y, z, z)) return;
  const int64_t o = cidx(x16, y, z, g);
  const uint4 t = *reinterpret_cast<const uint4*>(T + o);
  if ((t.x | t.y | t.z | t.w) == 0u) return;
  const uint4 e = *reinterpret_cast<const uint4*>(Ef + o);
  uint4 c = *reinterpret_cast<const uint4*>(C + o);
  c.x = (t.x & ~e.x) | (~t.x & c.x);
  c.y = (t.y & ~e.y) | (~t.y & c.y);
  c.z = (t.z & ~e.z) | (~t.z & c.z);
  c.w = (t.w & ~e.w) | (~t.w & c.w);
  *reinterpret_cast<uint4*>(C + o) = c;
}





// max clamped radius over the fine radius grid
__global__ void k_rmax(const int8_t* __restrict__ R, int64_t n, int* __restrict__ out) {
  int m = 2;
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * 16; i < n;
       i += (int64_t)gridDim.x * blockDim.x * 16) {
    const uint4 v = *reinterpret_cast<const uint4*>(R + i);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int s = (int)(int8_t)((w[j >> 2] >> (8 * (j & 3))) & 0xff);
      const int r = clamp_radius(s);
      m = r > m ? r : m;
    }
  }
  for (int o = 16; o > 0; o >>= 1) { const int t = __shfl_xor_sync(0xffffffffu, m, o); m = t > m ? t : m; }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// ---------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------

static inline int cdiv(int a, int b) { return (a + b - 1) / b; }

static int grid_stride_blocks(int64_t n, int threads, int sms) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)sms * 32;
  return (int)(b < cap ? b : cap);
}

// tile-need test by output box only (x and third coordinates in fine voxels
// or cells by the shifts)
static NeedMap roi_only(const CBox& b, int x_shift, int t_shift) {
  return NeedMap{nullptr, 0, 0, 0, x_shift, t_shift, 0, 0, 0, b};
}

// box grown by g cells along each axis flagged in `axes` (bit a), clamped
static CBox cbox_grow(const CBox& b, int g, int axes, const int dims[3]) {
  CBox r = b;
  for (int a = 0; a < 3; a++) {
    if ((axes >> a) & 1) {
      r.lo[a] = b.lo[a] - g;
      r.hi[a] = b.hi[a] + g;
    }
    r.lo[a] = r.lo[a] < 0 ? 0 : r.lo[a];
    r.hi[a] = r.hi[a] > dims[a] ? dims[a] : r.hi[a];
  }
  return r;
}

size_t close_workspace_bytes_box(int rx, int ry, int rz) {
  const size_t Nx = 2 * (size_t)rx, Ny = 2 * (size_t)ry, Nz = 2 * (size_t)rz, V = Nx * Ny * Nz;
  const size_t cells = (size_t)rx * ry * rz;
  // buf16 x2, buf8, HL1, HL2, Df, Eb, Ef, S, D, radius map, D and tag block maps + alignment slack
  return 2 * V * 2 + V + (size_t)rx * Ny * Nz * 2 + (size_t)rx * ry * Nz * 2 + 5 * cells + V / 4096 + 2 * (cells / 512) +
         17 * 256;
}

size_t close_workspace_bytes(int res) { return close_workspace_bytes_box(res, res, res); }

static inline uint8_t* carve(uint8_t*& p, size_t bytes) {
  uint8_t* r = p;
  p += (bytes + 255) & ~(size_t)255;
  return r;
}

// The closing's workspace, carved the same way by every entry point that
// works in it (launch_close and the parts that run before it).
struct CloseWs {
  uint16_t *buf16a, *buf16b, *HL1, *HL2;
  uint8_t *buf8, *Df, *Eb, *Ef, *S, *D, *rmap, *dmap, *tmap;
};

static CloseWs close_ws(const CloseArgs& a, int rx, int ry, int rz) {
  const size_t Nx = 2 * (size_t)rx, Ny = 2 * (size_t)ry, Nz = 2 * (size_t)rz, V = Nx * Ny * Nz;
  const size_t cells = (size_t)rx * ry * rz, blocks8 = cells / 512;
  uint8_t* p = a.workspace;
  CloseWs w;
  w.buf16a = reinterpret_cast<uint16_t*>(carve(p, V * 2));
  w.buf16b = reinterpret_cast<uint16_t*>(carve(p, V * 2));
  w.buf8 = carve(p, V);
  w.HL1 = reinterpret_cast<uint16_t*>(carve(p, (size_t)rx * Ny * Nz * 2));
  w.HL2 = reinterpret_cast<uint16_t*>(carve(p, (size_t)rx * ry * Nz * 2));
  w.Df = carve(p, cells);
  w.Eb = carve(p, cells);
  w.Ef = carve(p, cells);
  w.S = carve(p, cells);
  w.D = a.D_out != nullptr ? a.D_out : carve(p, cells);
  w.rmap = carve(p, V / 4096);
  w.dmap = carve(p, blocks8);
  w.tmap = carve(p, blocks8);
  return w;
}

uint8_t* close_ws_dilation(const CloseArgs& a) {
  const int rx = a.dims[0] > 0 ? a.dims[0] : a.res;
  const int ry = a.dims[0] > 0 ? a.dims[1] : a.res;
  const int rz = a.dims[0] > 0 ? a.dims[2] : a.res;
  return close_ws(a, rx, ry, rz).D;
}

// buf16a: first written by the dilation's passes or, when the dilation is
// done, by the erosion's x pass
uint8_t* close_ws_scratch(const CloseArgs& a, size_t* bytes) {
  const int rx = a.dims[0] > 0 ? a.dims[0] : a.res;
  const int ry = a.dims[0] > 0 ? a.dims[1] : a.res;
  const int rz = a.dims[0] > 0 ? a.dims[2] : a.res;
  const CloseWs w = close_ws(a, rx, ry, rz);
  if (bytes) *bytes = (size_t)(reinterpret_cast<uint8_t*>(w.buf16b) - reinterpret_cast<uint8_t*>(w.buf16a));
  return reinterpret_cast<uint8_t*>(w.buf16a);
}

uint16_t* close_ws_field(const CloseArgs& a) {
  const int rx = a.dims[0] > 0 ? a.dims[0] : a.res;
  const int ry = a.dims[0] > 0 ? a.dims[1] : a.res;
  const int rz = a.dims[0] > 0 ? a.dims[2] : a.res;
  return close_ws(a, rx, ry, rz).buf16b;
}

cudaError_t launch_close(const CloseArgs& a, cudaStream_t st, KernelCounter* kc) {
  const int rx = a.dims[0] > 0 ? a.dims[0] : a.res;
  const int ry = a.dims[0] > 0 ? a.dims[1] : a.res;
  const int rz = a.dims[0] > 0 ? a.dims[2] : a.res;
  if (rx % 16 != 0 || ry % 16 != 0 || rz % 16 != 0 || rx <= 0 || ry <= 0 || rz <= 0) return cudaErrorInvalidValue;
  const Dims g{rx, ry, rz};
  const int Nx = 2 * rx, Ny = 2 * ry, Nz = 2 * rz;
  const size_t cells = (size_t)rx * ry * rz;
  const CloseWs w = close_ws(a, rx, ry, rz);
  uint16_t* buf16a = w.buf16a;
  uint16_t* buf16b = w.buf16b;
  uint8_t* buf8 = w.buf8;
  uint16_t* HL1 = w.HL1;
  uint16_t* HL2 = w.HL2;
  uint8_t* Df = w.Df;
  uint8_t* Eb = w.Eb;
  uint8_t* Ef = w.Ef;
  uint8_t* S = w.S;
  uint8_t* D = w.D;
  uint8_t* rmap = w.rmap;
  const int mdx = rx / 8, mdy = ry / 8, mdz = rz / 8;
  uint8_t* dmap = w.dmap;
  uint8_t* tmap = w.tmap;  // 8^3-cell blocks holding refinement-tagged cells
  const int rmax = a.rmax;
  DataRes dr{{a.data_res[0], a.data_res[1], a.data_res[2]}};
  const bool exact = a.mode == 1;
  const RField RF{a.R, a.r_sy > 0 ? a.r_sy : (int64_t)Nx, a.r_sz > 0 ? a.r_sz : (int64_t)Nx * Ny};
  const RField RNONE{nullptr, 0, 0};
  // Output boxes of the passes (cells).  F: where the caller needs the
  // closing.  Working backwards: the erosion flags on F (centres) and F + 1
  // (lattice points, read by the neighbour test), the contour within the
  // erosion reach of those, the dilation one cell further (contour
  // neighbours) and its fine flags one more (forward 2x2x2 block); each
  // y (z) pass also within the window of the following pass.
  const int dims[3] = {rx, ry, rz};
  CBox F{{0, 0, 0}, {rx, ry, rz}};
  if (a.roi_hi[0] > 0)
    for (int k = 0; k < 3; k++) {
      F.lo[k] = a.roi_lo[k] < 0 ? 0 : a.roi_lo[k];
      F.hi[k] = a.roi_hi[k] > dims[k] ? dims[k] : a.roi_hi[k];
    }
  const int win = (rmax + 3) / 2 + 2;  // cells covering a pass window (rmax + 2 fine voxels) with rounding
  const CBox R_Ef = F, R_Eb = cbox_grow(F, 1, 7, dims);
  const CBox R_S = cbox_grow(F, win + 2, 7, dims), R_D = cbox_grow(R_S, 1, 7, dims), R_Df = cbox_grow(R_D, 1, 7, dims);
  const CBox B_dil_y = cbox_grow(R_Df, win, 4, dims), B_dil_x = cbox_grow(R_Df, win, 6, dims);
  const CBox B_ero_y = cbox_grow(R_Ef, win, 4, dims), B_erob_y = cbox_grow(R_Eb, win, 4, dims);
  const CBox B_ero_x = cbox_grow(R_Eb, win, 6, dims);
  // phase mode: the steps of phase a.phase only (see CloseArgs::phase)
  if (a.phase >= 0 && (a.edt != nullptr || !close_phase_ok(rmax, a.se) || a.group == nullptr))
    return cudaErrorInvalidValue;
  int at = 0;  // min-plus passes met so far
  auto here = [&]() { return a.phase < 0 || a.phase == at; };

  // ---- dilation ---- (skipped when the caller has put it in D already)
  if (!a.dilation_done) {
    const int dil_r = rmax + 1;  // "Safety Measure" radius + 1 (GMorpho.cu:2864)
    const int dcap = (a.se == 1 ? rmax + 2 : dil_r + 1) < 255 ? (a.se == 1 ? rmax + 2 : dil_r + 1) : 255;
    const uint32_t dil_cap = a.se == 1 ? (uint32_t)(rmax + 1) : (uint32_t)(dil_r * dil_r);
    const int dil_halo = dil_r + 1;
    const uint8_t* tile_map = nullptr;  // per-tile radius bounds of the dilation passes
    if (a.edt != nullptr) {
      // resident distance field: the dilation is its per-voxel threshold
      if (a.se != 0) return cudaErrorInvalidValue;
    } else if (a.R != nullptr && a.rmap_in != nullptr) {
      tile_map = a.rmap_in;  // built by the caller together with the radius bound
    } else if (a.R != nullptr) {
      if (here() && launch_radius_map(RF, Nx, Ny, Nz, rmap, nullptr, st, kc) != cudaSuccess)
        return cudaGetLastError();
      tile_map = rmap;
    }
    if (a.edt != nullptr) {
      GM_LAUNCH(kc, "k_dil_threshold", st,
                k_dil_threshold<<<quad_grid(g), dim3(64, 4), 0, st>>>(a.edt, a.e_sy, a.e_sz, RF, a.uniform_r, g,
                                                                      exact ? D : Df, R_Df));
    } else {
      if (!a.xpass_done && here() && launch_dil_pass_x(a.X, buf8, rx, ry, rz, dcap, B_dil_x, st, kc) != cudaSuccess)
        return cudaGetLastError();
      uint8_t* dst = exact ? D : Df;
      if ((a.ypass_done || a.zpass_done) && a.se != 0) return cudaErrorInvalidValue;
      if (dil_cap <= 32767) {
        bool ok = true;
        if (a.se == 1) {
          ok &= dpx_step<KERN_CUBE, uint8_t, 0>(a, at, buf8, buf16a, nullptr, Nx, Ny, Nz, 1, 0, dil_halo, dil_cap, RNONE,
                                                0, rx, ry, st, kc, "k_pass_dil_y", tile_map, dil_halo,
                                                roi_only(B_dil_y, 1, 1));
          ok &= dpx_step<KERN_CUBE, uint16_t, 1>(a, at, buf16a, nullptr, dst, Nx, Ny, Nz, 2, 0, dil_halo, dil_cap, RF,
                                                 a.uniform_r, rx, ry, st, kc, "k_pass_dil_z", tile_map, 0,
                                                 roi_only(R_Df, 1, 1));
        } else {
          if (!a.ypass_done)
            ok &= dpx_step<KERN_LAT, uint8_t, 0>(a, at, buf8, buf16a, nullptr, Nx, Ny, Nz, 1, 0, dil_halo, dil_cap,
                                                 RNONE, 0, rx, ry, st, kc, "k_pass_dil_y", tile_map, dil_halo,
                                                 roi_only(B_dil_y, 1, 1));
          else
            at++;
          if (!a.zpass_done)
            ok &= dpx_step<KERN_LAT, uint16_t, 1>(a, at, buf16a, nullptr, dst, Nx, Ny, Nz, 2, 0, dil_halo, dil_cap, RF,
                                                  a.uniform_r, rx, ry, st, kc, "k_pass_dil_z", tile_map, 0,
                                                  roi_only(R_Df, 1, 1));
          else
            at++;
        }
        if (!ok) return cudaErrorInvalidValue;
      } else {
        const int span = kTileOut + 2 * dil_halo;
        dim3 gy(cdiv(Nx, 32), cdiv(Ny, kTileOut), Nz);
        if (a.se == 1)
          GM_LAUNCH(kc, "k_axis_pass", st, k_axis_pass<KERN_CUBE, uint8_t><<<gy, dim3(32, kRows), span * 32 * 2, st>>>(
                                               buf8, buf16a, Nx, Ny, Nz, 1, 0, dil_halo, dil_cap));
        else
          GM_LAUNCH(kc, "k_axis_pass", st, k_axis_pass<KERN_LAT, uint8_t><<<gy, dim3(32, kRows), span * 32 * 2, st>>>(
                                               buf8, buf16a, Nx, Ny, Nz, 1, 0, dil_halo, dil_cap));
        dim3 gz(cdiv(Nx, 32), cdiv(Nz, kTileOut), Ny / 2);
        if (a.se == 1)
          GM_LAUNCH(kc, "k_final_z", st, k_final_z<KERN_CUBE, FIN_DIL><<<gz, dim3(32, 8), 2 * span * 32 * 2, st>>>(
                                             buf16a, dst, RF, a.uniform_r, rx, ry, rz, dil_halo, dil_cap));
        else
          GM_LAUNCH(kc, "k_final_z", st, k_final_z<KERN_LAT, FIN_DIL><<<gz, dim3(32, 8), 2 * span * 32 * 2, st>>>(
                                             buf16a, dst, RF, a.uniform_r, rx, ry, rz, dil_halo, dil_cap));
      }
    }
    if (!exact && here()) {
      GM_LAUNCH(kc, "k_dil_select", st,
                k_dil_select_z<<<dim3((g.x / 16 + 31) / 32, (g.y + 7) / 8, (g.z + kSelZ - 1) / kSelZ), dim3(32, 9), 0,
                                 st>>>(a.X, Df, D, g, dr, R_D));
    }
  } else {
    at += 2;  // the dilation's two passes
  }
  // ---- occupancy map of D (erosion outputs are needed on D only) ----
  if (here()) {
    const int nb = mdx * mdy * mdz;
    GM_LAUNCH(kc, "k_occ_map8", st, k_occ_map8<<<(nb + 7) / 8, 256, 0, st>>>(D, rx, ry, mdx, mdy, nb, dmap));
  }
  // ---- contour ----
  if (here()) {
    GM_LAUNCH(kc, "k_contour", st,
            k_contour_z<<<dim3((g.x / 16 + 31) / 32, (g.y + 7) / 8, (g.z + kConZ - 1) / kConZ), dim3(32, 10), 0, st>>>(
                D, S, g, exact ? 1 : 0, R_S));
    // (S holds the refinement tags after the erosion's x pass in GM_REF)
    if (a.S_out) cudaMemcpyAsync(a.S_out, S, cells, cudaMemcpyDeviceToDevice, st);
  }
  // ---- erosion ----
  {
    const uint32_t K = 4u * (uint32_t)((rmax - 1) * (rmax - 1));
    const int ehalo = rmax + 1;
    const int W = Nx >> 5;
    // bits, centre and lattice accumulators, compacted sites
    const size_t smem = sizeof(uint32_t) * (4 * (size_t)W + 4 * (size_t)Nx + 4 * (size_t)rx + 8 * (size_t)Nx);
    if (!here()) {
    } else if (W <= 64) {
      const size_t smem_w = kEroXWarps * ero_x_w_warp_bytes(rx);
      ensure_dynamic_smem(reinterpret_cast<const void*>(k_ero_pass_x_w), smem_w);
      const unsigned blocks = (unsigned)(((int64_t)ry * rz + kEroXWarps - 1) / kEroXWarps);
      GM_LAUNCH(kc, "k_ero_pass_x", st,
                k_ero_pass_x_w<<<blocks, 32 * kEroXWarps, smem_w, st>>>(S, RF, a.uniform_r, rx, ry, rz, ehalo, K,
                                                                        buf16a, HL1, B_ero_x));
    } else {
      ensure_dynamic_smem(reinterpret_cast<const void*>(k_ero_pass_x), smem);
      GM_LAUNCH(kc, "k_ero_pass_x", st,
                k_ero_pass_x<<<dim3(ry, rz), 256, smem, st>>>(S, RF, a.uniform_r, rx, ry, ehalo, K, buf16a, HL1,
                                                              B_ero_x));
    }
    if (K <= 32767) {
      const int gz = (ehalo + 1) / 2 + 1;  // cells covering the z window (ehalo fine voxels) of a z pass
      bool ok = true;
      if (exact) {
        // ero z needs its outputs on D grown by one cell, ero y its outputs
        // there and within the z window of it
        ok &= dpx_step<KERN_CEN2, uint16_t, 0>(a, at, buf16a, buf16b, nullptr, Nx, Ny, Nz, 1, 0, ehalo, K, RNONE, 0, rx,
                                               ry, st, kc, "k_pass_ero_y", nullptr, 0,
                                               NeedMap{dmap, mdx, mdy, mdz, 1, 1, 1, 1, 1 + gz, B_ero_y});
        ok &= dpx_step<KERN_CEN2, uint16_t, 2>(a, at, buf16b, nullptr, Ef, Nx, Ny, Nz, 2, 0, ehalo, K, RNONE, 0, rx, ry,
                                               st, kc, "k_pass_ero_z", nullptr, 0,
                                               NeedMap{dmap, mdx, mdy, mdz, 1, 1, 1, 1, 1, R_Ef});
      } else {
        // erob z needs its flags on D only, erob y within its z window
        ok &= dpx_step<KERN_LAT2, uint16_t, 0>(a, at, HL1, HL2, nullptr, rx, Ny, Nz, 1, 1, ehalo, K, RNONE, 0, rx, ry,
                                               st, kc, "k_pass_erob_y", nullptr, 0,
                                               NeedMap{dmap, mdx, mdy, mdz, 0, 1, 0, 0, gz, B_erob_y});
        ok &= dpx_step<KERN_LAT2, uint16_t, 3>(a, at, HL2, nullptr, Eb, rx, ry, Nz, 2, 1, ehalo, K, RNONE, 0, rx, ry,
                                               st, kc, "k_pass_erob_z", nullptr, 0,
                                               NeedMap{dmap, mdx, mdy, mdz, 0, 0, 0, 0, 0, R_Eb});
        // base erosion and refinement tags (the contour S is read by nobody
        // any more: it holds the tags), then the centre erosion only on the
        // blocks of tagged cells (ero y within the z window of them)
        if (here()) {
          cudaMemsetAsync(tmap, 0, (size_t)mdx * mdy * mdz, st);
          GM_LAUNCH(kc, "k_ero_tag", st,
                    k_ero_tag_z<<<dim3((g.x / 16 + 31) / 32, (g.y + 7) / 8, (g.z + kTagZ - 1) / kTagZ), dim3(32, 10), 0,
                                  st>>>(a.X, D, Eb, a.C_out, S, tmap, mdx, mdy, g, dr, F));
        }
        ok &= dpx_step<KERN_CEN2, uint16_t, 0>(a, at, buf16a, buf16b, nullptr, Nx, Ny, Nz, 1, 0, ehalo, K, RNONE, 0, rx,
                                               ry, st, kc, "k_pass_ero_y", nullptr, 0,
                                               NeedMap{tmap, mdx, mdy, mdz, 1, 1, 0, 0, gz, B_ero_y});
        ok &= dpx_step<KERN_CEN2, uint16_t, 2>(a, at, buf16b, nullptr, Ef, Nx, Ny, Nz, 2, 0, ehalo, K, RNONE, 0, rx, ry,
                                               st, kc, "k_pass_ero_z", nullptr, 0,
                                               NeedMap{tmap, mdx, mdy, mdz, 1, 1, 0, 0, 0, R_Ef});
        if (here())
          GM_LAUNCH(kc, "k_ero_fix", st, k_ero_fix16<<<grid16(g), dim3(32, 8), 0, st>>>(S, Ef, a.C_out, g, F));
      }
      if (!ok) return cudaErrorInvalidValue;
    } else {
      const int span = kTileOut + 2 * ehalo;
      dim3 gy(cdiv(Nx, 32), cdiv(Ny, kTileOut), Nz);
      GM_LAUNCH(kc, "k_axis_pass", st, k_axis_pass<KERN_CEN2, uint16_t><<<gy, dim3(32, kRows), span * 32 * 2, st>>>(
                                           buf16a, buf16b, Nx, Ny, Nz, 1, 0, ehalo, K));
      dim3 gz(cdiv(Nx, 32), cdiv(Nz, kTileOut), Ny / 2);
      GM_LAUNCH(kc, "k_final_z", st, k_final_z<KERN_CEN2, FIN_ERO><<<gz, dim3(32, 8), 2 * span * 32 * 2, st>>>(
                                         buf16b, Ef, RNONE, 0, rx, ry, rz, ehalo, K));
      if (!exact) {
        const int span_s = 2 * kTileOut + 2 * ehalo;
        dim3 gyb(cdiv(rx, 32), cdiv(ry, kTileOut), Nz);
        GM_LAUNCH(kc, "k_axis_pass", st, k_axis_pass<KERN_LAT2, uint16_t><<<gyb, dim3(32, kRows), span_s * 32 * 2, st>>>(
                                             HL1, HL2, rx, Ny, Nz, 1, 1, ehalo, K));
        dim3 gzb(cdiv(rx, 32), cdiv(rz, kTileOut), ry);
        GM_LAUNCH(kc, "k_final_z_base", st, k_final_z_base<<<gzb, dim3(32, kRows), span_s * 32 * 2, st>>>(
                                                HL2, Eb, rx, ry, rz, ehalo, K));
      }
    }
    if ((exact || K > 32767) && here())
      GM_LAUNCH(kc, "k_ero_select", st,
                k_ero_select16<<<grid16(g), dim3(32, 8), 0, st>>>(a.X, D, Eb, Ef, a.C_out, g, dr, exact ? 1 : 0, F));
  }
  return cudaGetLastError();
}

int close_phases(int mode) { return mode == 1 ? 5 : 7; }

bool close_phase_ok(int rmax, int se) {
  // the min-plus passes' saturation values fit 15 bits: the dilation's
  // (rmax + 1)^2 (sphere) or rmax + 1 (cube), the erosion's 4 (rmax - 1)^2
  const int r = clamp_radius(rmax);
  return (se == 1 || (r + 1) * (r + 1) <= 32767) && 4 * (r - 1) * (r - 1) <= 32767;
}

cudaError_t launch_edt(const uint8_t* X, int res, int rmax, uint8_t* workspace, uint16_t* E, cudaStream_t st,
                       KernelCounter* kc) {
  if (res % 16 != 0 || res <= 0 || rmax < 2 || rmax > 127) return cudaErrorInvalidValue;
  const int N = 2 * res;
  const size_t V = (size_t)N * N * N;
  uint8_t* p = workspace;
  uint16_t* buf16a = reinterpret_cast<uint16_t*>(carve(p, V * 2));
  carve(p, V * 2);
  uint8_t* buf8 = carve(p, V);
  // the sphere dilation's passes with the saturation of the largest radius
  // and no per-tile radius bound (every radius up to rmax may be asked)
  const int dil_r = rmax + 1, dil_halo = dil_r + 1, dcap = dil_r + 1;
  const uint32_t dil_cap = (uint32_t)(dil_r * dil_r);
  const RField RNONE{nullptr, 0, 0};
  if (launch_dil_pass_x(X, buf8, res, res, res, dcap, CBox{{0, 0, 0}, {res, res, res}}, st, kc) != cudaSuccess)
    return cudaGetLastError();
  launch_dpx<KERN_LAT, uint8_t, 0>(buf8, buf16a, nullptr, N, N, N, 1, 0, dil_halo, dil_cap, RNONE, 0, res, res, st,
                                   kc, "k_pass_dil_y");
  launch_dpx<KERN_LAT, uint16_t, 0>(buf16a, E, nullptr, N, N, N, 2, 0, dil_halo, dil_cap, RNONE, 0, res, res, st,
                                    kc, "k_pass_edt_z");
  return cudaGetLastError();
}

cudaError_t launch_close_xpass(const CloseArgs& a, cudaStream_t st, KernelCounter* kc) {
  const int rx = a.dims[0] > 0 ? a.dims[0] : a.res;
  const int ry = a.dims[0] > 0 ? a.dims[1] : a.res;
  const int rz = a.dims[0] > 0 ? a.dims[2] : a.res;
  if (rx % 16 != 0 || ry % 16 != 0 || rz % 16 != 0 || rx <= 0 || ry <= 0 || rz <= 0) return cudaErrorInvalidValue;
  uint8_t* buf8 = close_ws(a, rx, ry, rz).buf8;
  // saturation of the largest clamped radius (127): exact distances up to
  // 129, so any radius bound found later is covered
  return launch_dil_pass_x(a.X, buf8, rx, ry, rz, 129, CBox{{0, 0, 0}, {rx, ry, rz}}, st, kc);
}

cudaError_t launch_close_ypass(const CloseArgs& a, int z0, int z1, int r_bound, cudaStream_t st, KernelCounter* kc) {
  const int rx = a.dims[0] > 0 ? a.dims[0] : a.res;
  const int ry = a.dims[0] > 0 ? a.dims[1] : a.res;
  const int rz = a.dims[0] > 0 ? a.dims[2] : a.res;
  if (rx % 16 != 0 || ry % 16 != 0 || rz % 16 != 0 || rx <= 0 || ry <= 0 || rz <= 0 || a.se != 0 ||
      a.rmap_in == nullptr || z0 < 0 || z1 > rz || z0 >= z1)
    return cudaErrorInvalidValue;
  const int Nx = 2 * rx, Ny = 2 * ry, Nz = 2 * rz;
  const CloseWs w = close_ws(a, rx, ry, rz);
  uint16_t* buf16a = w.buf16a;
  uint8_t* buf8 = w.buf8;
  const int rb = clamp_radius(r_bound);
  const int dil_r = rb + 1, dil_halo = dil_r + 1;
  const uint32_t dil_cap = (uint32_t)(dil_r * dil_r);
  const RField RNONE{nullptr, 0, 0};
  launch_dpx<KERN_LAT, uint8_t, 0>(buf8, buf16a, nullptr, Nx, Ny, Nz, 1, 0, dil_halo, dil_cap, RNONE, 0, rx, ry, st,
                                   kc, "k_pass_dil_y", a.rmap_in, dil_halo,
                                   NeedMap{nullptr, 0, 0, 0, 1, 1, 0, 0, 0,
                                           CBox{{0, 0, 0}, {1 << 30, 1 << 30, 1 << 30}}, z0, z1 - z0});
  return cudaGetLastError();
}

cudaError_t launch_close_zpass(const CloseArgs& a, int z0, int z1, int r_bound, cudaStream_t st, KernelCounter* kc) {
  const int rx = a.dims[0] > 0 ? a.dims[0] : a.res;
  const int ry = a.dims[0] > 0 ? a.dims[1] : a.res;
  const int rz = a.dims[0] > 0 ? a.dims[2] : a.res;
  // whole output tiles (32 cells along z) only
  if (rx % 16 != 0 || ry % 16 != 0 || rz % 16 != 0 || rx <= 0 || ry <= 0 || rz <= 0 || a.se != 0 ||
      a.rmap_in == nullptr || a.R == nullptr || z0 < 0 || z1 > rz || z0 >= z1 || z0 % 32 != 0 || z1 % 32 != 0)
    return cudaErrorInvalidValue;
  const int Nx = 2 * rx, Ny = 2 * ry, Nz = 2 * rz;
  const CloseWs w = close_ws(a, rx, ry, rz);
  uint8_t* dst = a.mode == 1 ? w.D : w.Df;
  const int rb = clamp_radius(r_bound);
  const int dil_r = rb + 1, dil_halo = dil_r + 1;
  const uint32_t dil_cap = (uint32_t)(dil_r * dil_r);
  const RField RF{a.R, a.r_sy > 0 ? a.r_sy : (int64_t)Nx, a.r_sz > 0 ? a.r_sz : (int64_t)Nx * Ny};
  launch_dpx<KERN_LAT, uint16_t, 1>(w.buf16a, nullptr, dst, Nx, Ny, Nz, 2, 0, dil_halo, dil_cap, RF, a.uniform_r, rx,
                                    ry, st, kc, "k_pass_dil_z", a.rmap_in, 0,
                                    NeedMap{nullptr, 0, 0, 0, 1, 1, 0, 0, 0,
                                            CBox{{0, 0, 0}, {1 << 30, 1 << 30, 1 << 30}}, 0, 0, z0 / 32,
                                            (z1 - z0) / 32});
  return cudaGetLastError();
}

cudaError_t launch_contour(const uint8_t* D, uint8_t* S, int res, int exact, cudaStream_t st, KernelCounter* kc) {
  const Dims g{res, res, res};
  GM_LAUNCH(kc, "k_contour", st,
            k_contour_z<<<dim3((g.x / 16 + 31) / 32, (g.y + 7) / 8, (g.z + kConZ - 1) / kConZ), dim3(32, 10), 0, st>>>(
                D, S, g, exact, CBox{{0, 0, 0}, {res, res, res}}));
  return cudaGetLastError();
}

cudaError_t launch_rmax(const int8_t* R, int64_t n, int* d_out, int sms, cudaStream_t st, KernelCounter* kc) {
  cudaMemsetAsync(d_out, 0, sizeof(int), st);
  const int64_t vec = n / 16;
  int blocks = grid_stride_blocks(vec, 256, sms);
  if (blocks < 1) blocks = 1;
  GM_LAUNCH(kc, "k_rmax", st, k_rmax<<<blocks, 256, 0, st>>>(R, n, d_out));
  return cudaGetLastError();
}

}  // namespace gm
