// bvh.cu — linear BVH over fine voxels (reference row a18: BVH::
// BuildFromSEList, BuildSphereLeafNodes, BuildSphereInternalNodes,
// ComputeBottomUpSpheres, GMorpho::ErodeByBVH; GMorpho/BVH.cu:66-739,
// GMorpho/GMorpho.cu:8957-9401).
//
// Same construction as the reference (Morton-ordered leaves, Karras radix
// tree, bottom-up bounding volumes with one atomic counter per internal
// node), re-designed for exactness and for 2048^3 grids:
//   * leaves are enumerated directly in Morton order from the packed grid
//     (cells in Morton order, the eight children of a cell in child order,
//     which is the fine Morton order) - no sort;
//   * keys are 64-bit Morton codes (the reference's 30-bit codes overflow
//     beyond 1024 per axis);
//   * bounding volumes are integer boxes of the leaf voxels instead of float
//     spheres, so the pruning is exact and the query answers exactly
//     "is there a leaf voxel centre within distance < r of the query point".
#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

__device__ __forceinline__ uint64_t spread21(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}
__device__ __forceinline__ uint32_t gather21(uint64_t v) {
  v &= 0x1249249249249249ull;
  v = (v | (v >> 2)) & 0x10c30c30c30c30c3ull;
  v = (v | (v >> 4)) & 0x100f00f00f00f00full;
  v = (v | (v >> 8)) & 0x1f0000ff0000ffull;
  v = (v | (v >> 16)) & 0x1f00000000ffffull;
  v = (v | (v >> 32)) & 0x1fffffull;
  return (uint32_t)v;
}
__device__ __forceinline__ uint64_t morton64(uint32_t x, uint32_t y, uint32_t z) {
  return spread21(x) | (spread21(y) << 1) | (spread21(z) << 2);
}

// 16^3-cell bricks in Morton order: count the set fine voxels of each brick
__global__ void k_bvh_count(const uint8_t* __restrict__ g, int res, uint32_t* __restrict__ brick_cnt) {
  const int b = blockIdx.x;
  const int ox = (int)gather_bits3((uint32_t)b) * 16, oy = (int)gather_bits3((uint32_t)b >> 1) * 16,
            oz = (int)gather_bits3((uint32_t)b >> 2) * 16;
  uint32_t s = 0;
  for (int l = threadIdx.x; l < 4096; l += blockDim.x) {
    const int x = ox + (int)gather_bits3((uint32_t)l), y = oy + (int)gather_bits3((uint32_t)l >> 1),
              z = oz + (int)gather_bits3((uint32_t)l >> 2);
    s += __popc((uint32_t)g[cell_index(x, y, z, res)]);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ uint32_t ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += ws[w];
    brick_cnt[b] = t;
  }
}

// emit the leaves of each brick in Morton order (block = 256 threads, each
// thread 16 consecutive Morton cells)
__global__ void __launch_bounds__(256) k_bvh_emit(const uint8_t* __restrict__ g, int res,
                                                  const uint32_t* __restrict__ brick_off, uint64_t* __restrict__ keys) {
  const int b = blockIdx.x;
  const int ox = (int)gather_bits3((uint32_t)b) * 16, oy = (int)gather_bits3((uint32_t)b >> 1) * 16,
            oz = (int)gather_bits3((uint32_t)b >> 2) * 16;
  uint32_t cnt = 0;
  for (int i = 0; i < 16; i++) {
    const int l = threadIdx.x * 16 + i;
    cnt += __popc((uint32_t)g[cell_index(ox + (int)gather_bits3((uint32_t)l), oy + (int)gather_bits3((uint32_t)l >> 1),
                                         oz + (int)gather_bits3((uint32_t)l >> 2), res)]);
  }
  __shared__ uint32_t wt[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) wt[wid] = x;
  __syncthreads();
  uint32_t pre = 0;
  for (int w = 0; w < wid; w++) pre += wt[w];
  uint32_t pos = brick_off[b] + pre + x - cnt;
  for (int i = 0; i < 16; i++) {
    const int l = threadIdx.x * 16 + i;
    const int cx = ox + (int)gather_bits3((uint32_t)l), cy = oy + (int)gather_bits3((uint32_t)l >> 1),
              cz = oz + (int)gather_bits3((uint32_t)l >> 2);
    const uint32_t v = g[cell_index(cx, cy, cz, res)];
    for (int k = 0; k < 8; k++)
      if ((v >> k) & 1u) keys[pos++] = morton64(2 * cx + (k & 1), 2 * cy + ((k >> 1) & 1), 2 * cz + (k >> 2));
  }
}

__device__ __forceinline__ int delta64(const uint64_t* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  return __clzll((long long)(keys[i] ^ keys[j]));
}

// Karras (2012) radix tree over sorted unique keys: internal node i spans a
// key range and splits it at the highest differing bit.  Child indices:
// >= 0 internal, < 0 leaf (~index).
__global__ void k_bvh_internal(const uint64_t* __restrict__ keys, int n, int2* __restrict__ child,
                               int* __restrict__ parent) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
    const int d = delta64(keys, n, i, i + 1) > delta64(keys, n, i, i - 1) ? 1 : -1;
    const int dmin = delta64(keys, n, i, i - d);
    int lmax = 2;
    while (delta64(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t > 0; t /= 2)
      if (delta64(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta64(keys, n, i, j);
    int s = 0;
    for (int div = 2;; div *= 2) {
      const int t = (l + div - 1) / div;
      if (delta64(keys, n, i, i + (s + t) * d) > dnode) s += t;
      if (t <= 1) break;
    }
    const int gamma = i + s * d + (d < 0 ? -1 : 0);
    const int lo = i < j ? i : j, hi = i < j ? j : i;
    const int left = lo == gamma ? ~gamma : gamma;
    const int right = hi == gamma + 1 ? ~(gamma + 1) : gamma + 1;
    child[i] = make_int2(left, right);
    if (left >= 0) parent[left] = i;
    else parent[(n - 1) + ~left] = i;
    if (right >= 0) parent[right] = i;
    else parent[(n - 1) + ~right] = i;
  }
}

struct __align__(16) Box16 {
  short lo[3], hi[3];
  int pad;
};

// boxes written by other threads are read around L1 (it is not coherent)
__device__ __forceinline__ Box16 load_box_cg(const Box16* p) {
  const uint4 v = __ldcg(reinterpret_cast<const uint4*>(p));
  Box16 b;
  *reinterpret_cast<uint4*>(&b) = v;
  return b;
}

// bottom-up boxes: the second child to arrive at a node merges (one
// atomic counter per internal node, as ComputeBottomUpSpheres does)
__global__ void k_bvh_boxes(const uint64_t* __restrict__ keys, int n, const int2* __restrict__ child,
                            const int* __restrict__ parent, unsigned int* __restrict__ counter,
                            Box16* __restrict__ box) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    const short x = (short)gather21(k), y = (short)gather21(k >> 1), z = (short)gather21(k >> 2);
    Box16 lb;
    lb.pad = 0;
    lb.lo[0] = lb.hi[0] = x;
    lb.lo[1] = lb.hi[1] = y;
    lb.lo[2] = lb.hi[2] = z;
    box[(n - 1) + i] = lb;
    if (n == 1) continue;
    __threadfence();
    int node = parent[(n - 1) + i];
    while (node >= 0) {
      if (atomicAdd(counter + node, 1u) == 0) break;  // first arrival: the sibling finishes
      __threadfence();
      const int2 c = child[node];
      const Box16 a = load_box_cg(box + (c.x >= 0 ? c.x : (n - 1) + ~c.x));
      const Box16 b = load_box_cg(box + (c.y >= 0 ? c.y : (n - 1) + ~c.y));
      Box16 m;
      m.pad = 0;
      for (int t = 0; t < 3; t++) {
        m.lo[t] = a.lo[t] < b.lo[t] ? a.lo[t] : b.lo[t];
        m.hi[t] = a.hi[t] > b.hi[t] ? a.hi[t] : b.hi[t];
      }
      box[node] = m;
      __threadfence();
      node = node == 0 ? -1 : parent[node];
    }
  }
}

// squared distance (half-voxel units) from point q2 to the box of voxel
// centres [2 lo + 1, 2 hi + 1]
__device__ __forceinline__ int64_t box_sqd2(const Box16& b, const int q2[3]) {
  int64_t s = 0;
  for (int t = 0; t < 3; t++) {
    const int lo = 2 * b.lo[t] + 1, hi = 2 * b.hi[t] + 1;
    const int d = q2[t] < lo ? lo - q2[t] : (q2[t] > hi ? q2[t] - hi : 0);
    s += (int64_t)d * d;
  }
  return s;
}

// 1 when some leaf voxel centre lies at distance < r of the query (queries
// in half-voxel units).  Depth-first with a bounded stack; a traversal that
// would overflow it reports 2 (never silently drops a subtree).
__device__ int bvh_hit(const int2* __restrict__ child, const Box16* __restrict__ box, int n, const int q2[3],
                       int64_t r2x4) {
  if (n == 0) return 0;
  if (n == 1) return box_sqd2(box[0], q2) < r2x4 ? 1 : 0;
  int stack[96];
  int sp = 0;
  int node = 0;
  if (box_sqd2(box[0], q2) >= r2x4) return 0;
  while (true) {
    const int2 c = child[node];
    const int ids[2] = {c.x, c.y};
    int next = -1;
    for (int s = 0; s < 2; s++) {
      const int id = ids[s];
      const int bi = id >= 0 ? id : (n - 1) + ~id;
      if (box_sqd2(box[bi], q2) >= r2x4) continue;
      if (id < 0) return 1;  // a leaf box is the voxel centre itself
      if (next < 0) next = id;
      else {
        if (sp >= 96) return 2;
        stack[sp++] = id;
      }
    }
    if (next >= 0) node = next;
    else if (sp > 0) node = stack[--sp];
    else return 0;
  }
}

__global__ void k_bvh_query(const int2* __restrict__ child, const Box16* __restrict__ box, int n,
                            const int32_t* __restrict__ q2, int64_t nq, int64_t r2x4, uint8_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x) {
    const int q[3] = {q2[3 * i], q2[3 * i + 1], q2[3 * i + 2]};
    out[i] = (uint8_t)bvh_hit(child, box, n, q, r2x4);
  }
}

// ErodeByBVH fine predicate (GMorpho.cu:8957-9060): a voxel of D in a cell
// with D != 0 and X != 0xff inside data_res is removed when a leaf centre is
// at distance < r of its centre.
__global__ void k_bvh_erode(const int2* __restrict__ child, const Box16* __restrict__ box, int n,
                            const uint8_t* __restrict__ X, const uint8_t* __restrict__ D, int res, int dx, int dy,
                            int dz, int64_t r2x4, uint8_t* __restrict__ C, int* __restrict__ overflow) {
  const int64_t total = (int64_t)res * res * res;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < total; c += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(c % res), y = (int)((c / res) % res), z = (int)(c / ((int64_t)res * res));
    const uint8_t d = D[c];
    uint8_t out = d;
    if (d != 0 && X[c] != 0xff && x < dx && y < dy && z < dz) {
      for (int k = 0; k < 8; k++) {
        if (!((d >> k) & 1)) continue;
        const int q[3] = {2 * (2 * x + (k & 1)) + 1, 2 * (2 * y + ((k >> 1) & 1)) + 1, 2 * (2 * z + (k >> 2)) + 1};
        const int h = bvh_hit(child, box, n, q, r2x4);
        if (h == 2) atomicExch(overflow, 1);
        if (h) out &= (uint8_t)~(1u << k);
      }
    }
    C[c] = out;
  }
}

// ------------------------------------------------------------------ host

struct BvhDev {
  int n = 0;
  uint64_t* keys = nullptr;
  int2* child = nullptr;
  int* parent = nullptr;
  unsigned int* counter = nullptr;
  Box16* box = nullptr;
};

static int blocks(int64_t n, int t) {
  int64_t b = (n + t - 1) / t;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

cudaError_t bvh_build(const uint8_t* grid, int res, void** handle, uint32_t* scratch_bricks, int* n_out,
                      cudaStream_t st, KernelCounter* kc) {
  const int nb = (int)((int64_t)res * res * res / 4096);
  GM_LAUNCH(kc, "k_bvh_count", st, k_bvh_count<<<nb, 256, 0, st>>>(grid, res, scratch_bricks));
  // exclusive scan of the brick counts on the host side of a small copy
  uint32_t* h = new uint32_t[nb + 1];
  cudaMemcpyAsync(h, scratch_bricks, sizeof(uint32_t) * nb, cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { delete[] h; return e; }
  uint64_t run = 0;
  for (int b = 0; b < nb; b++) { const uint32_t v = h[b]; h[b] = (uint32_t)run; run += v; }
  if (run > 0x7fffffff) { delete[] h; return cudaErrorInvalidValue; }
  const int n = (int)run;
  cudaMemcpyAsync(scratch_bricks, h, sizeof(uint32_t) * nb, cudaMemcpyHostToDevice, st);
  e = cudaStreamSynchronize(st);
  delete[] h;
  if (e != cudaSuccess) return e;
  BvhDev* b = new BvhDev();
  b->n = n;
  const int64_t nn = n > 0 ? n : 1;
  if ((e = cudaMalloc(&b->keys, sizeof(uint64_t) * nn)) != cudaSuccess ||
      (e = cudaMalloc(&b->child, sizeof(int2) * nn)) != cudaSuccess ||
      (e = cudaMalloc(&b->parent, sizeof(int) * 2 * nn)) != cudaSuccess ||
      (e = cudaMalloc(&b->counter, sizeof(unsigned int) * nn)) != cudaSuccess ||
      (e = cudaMalloc(&b->box, sizeof(Box16) * 2 * nn)) != cudaSuccess) {
    cudaFree(b->keys); cudaFree(b->child); cudaFree(b->parent); cudaFree(b->counter); cudaFree(b->box);
    delete b;
    return e;
  }
  if (n > 0) {
    GM_LAUNCH(kc, "k_bvh_emit", st, k_bvh_emit<<<nb, 256, 0, st>>>(grid, res, scratch_bricks, b->keys));
    cudaMemsetAsync(b->counter, 0, sizeof(unsigned int) * nn, st);
    cudaMemsetAsync(b->parent, 0xff, sizeof(int) * 2 * nn, st);
    if (n > 1) GM_LAUNCH(kc, "k_bvh_internal", st, k_bvh_internal<<<blocks(n - 1, 256), 256, 0, st>>>(b->keys, n, b->child, b->parent));
    GM_LAUNCH(kc, "k_bvh_boxes", st, k_bvh_boxes<<<blocks(n, 256), 256, 0, st>>>(b->keys, n, b->child, b->parent, b->counter, b->box));
  }
  *handle = b;
  *n_out = n;
  return cudaGetLastError();
}

void bvh_free(void* handle) {
  BvhDev* b = static_cast<BvhDev*>(handle);
  if (!b) return;
  cudaFree(b->keys); cudaFree(b->child); cudaFree(b->parent); cudaFree(b->counter); cudaFree(b->box);
  delete b;
}

cudaError_t bvh_query(const void* handle, const int32_t* q2, int64_t nq, int radius, uint8_t* out, cudaStream_t st,
                      KernelCounter* kc) {
  const BvhDev* b = static_cast<const BvhDev*>(handle);
  const int64_t r2x4 = 4ll * radius * radius;
  if (nq > 0)
    GM_LAUNCH(kc, "k_bvh_query", st,
              k_bvh_query<<<blocks(nq, 128), 128, 0, st>>>(b->child, b->box, b->n, q2, nq, r2x4, out));
  return cudaGetLastError();
}

cudaError_t bvh_erode(const void* handle, const uint8_t* X, const uint8_t* D, int res, const int* data_res,
                      int radius, uint8_t* C, int* d_overflow, cudaStream_t st, KernelCounter* kc) {
  const BvhDev* b = static_cast<const BvhDev*>(handle);
  const int64_t r2x4 = 4ll * radius * radius;
  const int64_t cells = (int64_t)res * res * res;
  cudaMemsetAsync(d_overflow, 0, sizeof(int), st);
  GM_LAUNCH(kc, "k_bvh_erode", st,
            k_bvh_erode<<<blocks(cells, 128), 128, 0, st>>>(b->child, b->box, b->n, X, D, res, data_res[0],
                                                             data_res[1], data_res[2], r2x4, C, d_overflow));
  return cudaGetLastError();
}

int bvh_size(const void* handle) { return handle ? static_cast<const BvhDev*>(handle)->n : 0; }

cudaError_t bvh_keys(const void* handle, uint64_t* out, cudaStream_t st) {
  const BvhDev* b = static_cast<const BvhDev*>(handle);
  if (b->n > 0) return cudaMemcpyAsync(out, b->keys, sizeof(uint64_t) * b->n, cudaMemcpyDeviceToDevice, st);
  return cudaSuccess;
}

}  // namespace gm
