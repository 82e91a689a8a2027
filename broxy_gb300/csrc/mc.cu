// mc.cu — contour marching cubes and mesh normals (reference rows a12..a16:
// Grid::ComputeContourMCM, ComputeMCMData/CompactMCMData, SplatIndices/
// BuildNeighbors, MarchingCubesMesher::createMesh3D, ComputeMeshNormals,
// BilateralMeshFiltering; GMorpho/Grid.cu:1329-1462, 1873-1973,
// GMorpho/GMorpho.cu:6109-6496, 6498-6620, 6814-7001,
// GMorpho/MarchingCubesMesher.cu:1297-1618).
//
// Emission order equals the reference's: base cells in Morton order (the
// reference sorts its contour list by 30-bit Morton code), eight sub-cubes
// per cell in child order, non-empty cubes compacted, owned edges 0, 3, 8
// numbered in that order.  Instead of a sort, cells are visited directly in
// Morton order: a 16^3 brick of cells is one contiguous 4096-code Morton
// range, so one block per brick with an in-block scan and a scan of the
// brick totals gives every cell its output offsets.  Instead of the 4V-byte
// splat map, a neighbour cube's vertex offset is its cell's offset (one u32
// per cell) plus an in-cell prefix recomputed from the grid.
#include "gm_common.cuh"
#include "gm_internal.h"
#include "mc_tables.inc"

namespace gm {

__constant__ uint64_t c_tri_packed[256] = GM_MC_TRI_PACKED_INIT;
__constant__ uint8_t c_tri_count[256] = GM_MC_TRI_COUNT_INIT;
__constant__ uint8_t c_tri_len[256] = GM_MC_TRI_LEN_INIT;

// Edge mask of an MC cube value, derived from the corner order v0..v7 =
// 000,100,110,010,001,101,111,011 and the edge list (0,1)(1,2)(2,3)(3,0)
// (4,5)(5,6)(6,7)(7,4)(0,4)(1,5)(2,6)(3,7).
__device__ __forceinline__ int edge_mask(int v) {
  const int x = v ^ (v >> 1);
  const int e3 = (v ^ (v >> 3)) & 1;
  const int e7 = ((v >> 7) ^ (v >> 4)) & 1;
  return (x & 7) | (e3 << 3) | (((x >> 4) & 7) << 4) | (e7 << 7) | (((v ^ (v >> 4)) & 0xF) << 8);
}
__device__ __forceinline__ int nv_owned(int em) { return (em & 1) + ((em >> 3) & 1) + ((em >> 8) & 1); }

constexpr int kBrick = 16;               // cells per brick edge
constexpr int kTileE = kBrick + 2;       // tile edge (halo 2 for neighbour cells)
constexpr int kTileP = 32;               // tile row pitch (bytes): rows are one 16-byte and one 2-byte store
constexpr int kTileCells = kTileP * kTileE * kTileE;
__device__ __forceinline__ int tix(int x, int y, int z) { return x + kTileP * (y + kTileE * z); }
constexpr int kCellsPerBrick = kBrick * kBrick * kBrick;
constexpr int kMcThreads = 256;
constexpr int kCellsPerThread = kCellsPerBrick / kMcThreads;

__device__ __forceinline__ void brick_origin(int b, int& ox, int& oy, int& oz) {
  ox = (int)gather_bits3((uint32_t)b) * kBrick;
  oy = (int)gather_bits3((uint32_t)b >> 1) * kBrick;
  oz = (int)gather_bits3((uint32_t)b >> 2) * kBrick;
}

// grid dimensions in cells (x, y, z); x-fastest
struct GDims { int x, y, z; };
__device__ __forceinline__ int64_t gidx(int x, int y, int z, GDims d) { return idx3(x, y, z, d.x, d.y); }

// Loads the tile (cells o .. o + 17 per axis, zero outside the grid) and
// tells (block-uniformly) whether it can hold a mixed cube: a tile whose
// bytes are all 0x00 or all 0xff has none.  One row (18 cells along x) is
// a 16-byte and a 2-byte load: bricks start at multiples of 16 cells and
// grid edges are multiples of 16, so a row is either inside the grid up to
// cell o + 15 or outside, and so are cells o + 16, o + 17.
__device__ bool load_tile_mixed(const uint8_t* __restrict__ C, GDims d, int ox, int oy, int oz, uint8_t* tile) {
  int seen0 = 0, seen1 = 0, part = 0;
  for (int row = threadIdx.x; row < kTileE * kTileE; row += blockDim.x) {
    const int ly = row % kTileE, lz = row / kTileE;
    const int y = oy + ly, z = oz + lz;
    uint4 q = make_uint4(0u, 0u, 0u, 0u);
    uint32_t h = 0u;
    if (y < d.y && z < d.z && ox < d.x) {
      q = *reinterpret_cast<const uint4*>(C + gidx(ox, y, z, d));
      if (ox + kBrick < d.x) h = *reinterpret_cast<const uint16_t*>(C + gidx(ox + kBrick, y, z, d));
    }
    uint8_t* trow = tile + kTileP * row;
    *reinterpret_cast<uint4*>(trow) = q;
    *reinterpret_cast<uint16_t*>(trow + kBrick) = (uint16_t)h;
    // the two halo bytes, repeated to fill a word (repeats change no test)
    const uint32_t w[5] = {q.x, q.y, q.z, q.w, h | (h << 16)};
#pragma unroll
    for (int k = 0; k < 5; k++) {
      const uint32_t z4 = __vcmpeq4(w[k], 0u), f4 = __vcmpeq4(w[k], 0xffffffffu);
      seen0 |= z4 != 0u;
      seen1 |= f4 != 0u;
      part |= (~(z4 | f4)) != 0u;
    }
  }
  const int mixed = __syncthreads_or(part | (seen0 & seen1));
  if (mixed) return true;
  // a block may have seen only zeros while another saw only full bytes
  return __syncthreads_or(seen0) && __syncthreads_or(seen1);
}

// The eight MC cube values of cell (local lx,ly,lz): cube k has its min
// corner at fine voxel 2c + o_k; value bit j = occupancy of corner j
// (ComputeMCMData, GMorpho.cu:6146-6232).
__device__ __forceinline__ void cube_values(const uint8_t* tile, int lx, int ly, int lz, int vals[8]) {
  uint32_t b27 = 0;
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const uint8_t cell = tile[tix(lx + (i >> 1), ly + (j >> 1), lz + (k >> 1))];
        const uint32_t bit = (cell >> ((i & 1) + 2 * (j & 1) + 4 * (k & 1))) & 1u;
        b27 |= bit << (i + 3 * j + 9 * k);
      }
#pragma unroll
  for (int s = 0; s < 8; s++) {
    const int ox = s & 1, oy = (s >> 1) & 1, oz = s >> 2;
    const int b = ox + 3 * oy + 9 * oz;
    // corners 000,100,110,010,001,101,111,011 -> offsets in the 27-cube
    int v = 0;
    v |= ((b27 >> (b + 0)) & 1) << 0;
    v |= ((b27 >> (b + 1)) & 1) << 1;
    v |= ((b27 >> (b + 4)) & 1) << 2;
    v |= ((b27 >> (b + 3)) & 1) << 3;
    v |= ((b27 >> (b + 9)) & 1) << 4;
    v |= ((b27 >> (b + 10)) & 1) << 5;
    v |= ((b27 >> (b + 13)) & 1) << 6;
    v |= ((b27 >> (b + 12)) & 1) << 7;
    vals[s] = v;
  }
}

// The MC value of sub-cube s of cell (lx, ly, lz) alone (cube_values()[s]).
__device__ __forceinline__ int cube_value(const uint8_t* tile, int lx, int ly, int lz, int s) {
  const int fx = 2 * lx + (s & 1), fy = 2 * ly + ((s >> 1) & 1), fz = 2 * lz + (s >> 2);
  int v = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    // corners 000, 100, 110, 010, 001, 101, 111, 011
    const int x = fx + (((c + 1) >> 1) & 1), y = fy + ((c >> 1) & 1), z = fz + (c >> 2);
    const uint32_t cell = tile[tix(x >> 1, y >> 1, z >> 1)];
    v |= (int)((cell >> ((x & 1) + 2 * (y & 1) + 4 * (z & 1))) & 1u) << c;
  }
  return v;
}

// True when the 2x2x2 block of cells c .. c+1 is all empty or all full: then
// none of the eight sub-cubes of c is mixed (cheap test before cube_values).
__device__ __forceinline__ bool cell_uniform(const uint8_t* tile, int lx, int ly, int lz) {
  uint32_t o = 0, a = 0xffu;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const uint32_t v = tile[tix(lx + (k & 1), ly + ((k >> 1) & 1), lz + (k >> 2))];
    o |= v;
    a &= v;
  }
  return o == 0u || a == 0xffu;
}

// Tagging / emission window of one meshing run.  A whole grid is its own
// window: off = 0, gdim = its size, tag and emit boxes = the whole grid.  The edit
// server meshes the dirty box of a crop: the crop's cells sit at global
// cells off + local, the border rule uses the global resolution, cubes are
// tagged (own vertices) in the dirty box plus one cell on the + side (the
// neighbour cubes whose edges the box's triangles use), and triangles come
// from the dirty box only.
struct McWin {
  int off[3];
  int gdim[3];         // global grid (cells): cubes of cells outside [1, gdim-2] are never tagged
  int tlo[3], thi[3];  // local cells whose cubes may be tagged, [lo, hi)
  int elo[3], ehi[3];  // local cells whose cubes emit triangles, [lo, hi)
};

// cells outside [1, gres-2]^3 are never tagged (TagVoxelsContourMCM,
// Grid.cu:1334-1340)
__device__ __forceinline__ bool win_tag(const McWin& w, int x, int y, int z) {
  const int gx = x + w.off[0], gy = y + w.off[1], gz = z + w.off[2];
  return gx >= 1 && gy >= 1 && gz >= 1 && gx <= w.gdim[0] - 2 && gy <= w.gdim[1] - 2 && gz <= w.gdim[2] - 2 &&
         x >= w.tlo[0] && y >= w.tlo[1] && z >= w.tlo[2] && x < w.thi[0] && y < w.thi[1] && z < w.thi[2];
}
__device__ __forceinline__ bool win_emit(const McWin& w, int x, int y, int z) {
  return x >= w.elo[0] && y >= w.elo[1] && z >= w.elo[2] && x < w.ehi[0] && y < w.ehi[1] && z < w.ehi[2];
}
// block-uniform: does the 16^3 brick at (ox, oy, oz) meet the tag box?
__device__ __forceinline__ bool brick_live(const McWin& w, int ox, int oy, int oz) {
  return ox < w.thi[0] && oy < w.thi[1] && oz < w.thi[2] && ox + kBrick > w.tlo[0] && oy + kBrick > w.tlo[1] &&
         oz + kBrick > w.tlo[2];
}

// mixed-cube mask of a cell (0 when the cell is not tagged)
__device__ __forceinline__ int mixed_mask(const int vals[8], bool tagged) {
  if (!tagged) return 0;
  int m = 0;
#pragma unroll
  for (int s = 0; s < 8; s++) m |= (vals[s] != 0 && vals[s] != 255) ? (1 << s) : 0;
  return m;
}

struct CellCounts {
  uint32_t cubes, verts, tris, n91;
};

__device__ __forceinline__ CellCounts cell_counts(const int vals[8], int mask) {
  CellCounts c{0, 0, 0, 0};
#pragma unroll
  for (int s = 0; s < 8; s++) {
    if (!((mask >> s) & 1)) continue;
    c.cubes += 1;
    c.verts += nv_owned(edge_mask(vals[s]));
    c.tris += c_tri_count[vals[s]];
    c.n91 += c_tri_len[vals[s]] > c_tri_count[vals[s]] ? 1 : 0;
  }
  return c;
}

__device__ __forceinline__ void local_coords(int l, int& lx, int& ly, int& lz) {
  lx = (int)gather_bits3((uint32_t)l);
  ly = (int)gather_bits3((uint32_t)l >> 1);
  lz = (int)gather_bits3((uint32_t)l >> 2);
}

// block-wide exclusive scan of 4 counters (256 threads)
__device__ __forceinline__ CellCounts block_exclusive_scan(CellCounts v, CellCounts& total) {
  __shared__ uint32_t warp_tot[4][kMcThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t a[4] = {v.cubes, v.verts, v.tris, v.n91};
  uint32_t inc[4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    uint32_t x = a[c];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    inc[c] = x;
    if (lane == 31) warp_tot[c][wid] = x;
  }
  __syncthreads();
  uint32_t wpre[4] = {0, 0, 0, 0}, tot[4] = {0, 0, 0, 0};
#pragma unroll
  for (int c = 0; c < 4; c++)
    for (int w = 0; w < kMcThreads / 32; w++) {
      if (w < wid) wpre[c] += warp_tot[c][w];
      tot[c] += warp_tot[c][w];
    }
  __syncthreads();
  total = CellCounts{tot[0], tot[1], tot[2], tot[3]};
  return CellCounts{wpre[0] + inc[0] - a[0], wpre[1] + inc[1] - a[1], wpre[2] + inc[2] - a[2],
                    wpre[3] + inc[3] - a[3]};
}

// block-wide exclusive scan of one counter (256 threads); total in `total`
__device__ __forceinline__ uint32_t block_scan1(uint32_t v, uint32_t& total) {
  __shared__ uint32_t wt[kMcThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) wt[wid] = x;
  __syncthreads();
  uint32_t pre = 0, tot = 0;
#pragma unroll
  for (int k = 0; k < kMcThreads / 32; k++) {
    pre += k < wid ? wt[k] : 0u;
    tot += wt[k];
  }
  __syncthreads();
  total = tot;
  return pre + x - v;
}

// The brick's own cells that may hold a tagged mixed cube (not uniform,
// inside the tag window), in Morton order, into list[]; returns how many
// (block-uniform).  The cube work then runs over this list with every lane
// busy, instead of each thread walking its 16 cells and the warp taking the
// slow path whenever one lane needs it.
__device__ int brick_candidates(const uint8_t* tile, const McWin& w, int ox, int oy, int oz, uint16_t* list) {
  uint32_t mask = 0;
#pragma unroll 4
  for (int i = 0; i < kCellsPerThread; i++) {
    const int l = threadIdx.x * kCellsPerThread + i;
    int lx, ly, lz;
    local_coords(l, lx, ly, lz);
    if (!cell_uniform(tile, lx, ly, lz) && win_tag(w, ox + lx, oy + ly, oz + lz)) mask |= 1u << i;
  }
  uint32_t total;
  uint32_t k = block_scan1(__popc(mask), total);
  while (mask) {
    const int i = __ffs(mask) - 1;
    mask &= mask - 1;
    list[k++] = (uint16_t)(threadIdx.x * kCellsPerThread + i);
  }
  __syncthreads();
  return (int)total;
}

__global__ void __launch_bounds__(kMcThreads, 5) k_mc_count(const uint8_t* __restrict__ C, GDims gd, McWin w,
                                                          uint32_t* __restrict__ brick_tot) {
  __shared__ __align__(16) uint8_t tile[kTileCells];
  __shared__ uint16_t list[kCellsPerBrick];
  int ox, oy, oz;
  brick_origin(blockIdx.x, ox, oy, oz);
  if (!brick_live(w, ox, oy, oz) || !load_tile_mixed(C, gd, ox, oy, oz, tile)) {
    if (threadIdx.x < 4) brick_tot[4 * blockIdx.x + threadIdx.x] = 0;
    return;
  }
  const int nc = brick_candidates(tile, w, ox, oy, oz, list);
  CellCounts acc{0, 0, 0, 0};
  for (int j = threadIdx.x; j < nc; j += blockDim.x) {
    int lx, ly, lz;
    local_coords(list[j], lx, ly, lz);
    int vals[8];
    cube_values(tile, lx, ly, lz, vals);
    const int m = mixed_mask(vals, true);
    if (!m) continue;
    const CellCounts c = cell_counts(vals, m);
    acc.cubes += c.cubes; acc.verts += c.verts;
    if (win_emit(w, ox + lx, oy + ly, oz + lz)) { acc.tris += c.tris; acc.n91 += c.n91; }
  }
  CellCounts tot;
  block_exclusive_scan(acc, tot);
  if (threadIdx.x == 0) {
    brick_tot[4 * blockIdx.x + 0] = tot.cubes;
    brick_tot[4 * blockIdx.x + 1] = tot.verts;
    brick_tot[4 * blockIdx.x + 2] = tot.tris;
    brick_tot[4 * blockIdx.x + 3] = tot.n91;
  }
}

// Exclusive scan of the four brick counters, in place, totals at index nb:
// chunks of 1024 bricks, one block each.  k_brick_sums leaves each chunk's
// sums after the counters (index nb + 1 + chunk); k_scan_bricks adds the
// sums of the chunks before its own and scans its chunk (16-byte loads).
constexpr int kBrickChunk = 1024;

__device__ __forceinline__ uint4 add4(uint4 a, uint4 b) { return make_uint4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ uint4 shfl_up4(uint4 v, int o) {
  return make_uint4(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o),
                    __shfl_up_sync(0xffffffffu, v.z, o), __shfl_up_sync(0xffffffffu, v.w, o));
}
__device__ __forceinline__ uint4 shfl4(uint4 v, int src) {
  return make_uint4(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
                    __shfl_sync(0xffffffffu, v.z, src), __shfl_sync(0xffffffffu, v.w, src));
}
// inclusive scan over the block (1024 threads); *total = the block's sum
__device__ __forceinline__ uint4 block_incl_scan4(uint4 v, uint4* total) {
  __shared__ uint4 warp_tot[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint4 t = shfl_up4(v, o);
    if (lane >= o) v = add4(v, t);
  }
  if (lane == 31) warp_tot[wid] = v;
  __syncthreads();
  if (wid == 0) {
    uint4 w = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint4 t = shfl_up4(w, o);
      if (lane >= o) w = add4(w, t);
    }
    warp_tot[lane] = w;
  }
  __syncthreads();
  if (wid > 0) v = add4(v, warp_tot[wid - 1]);
  *total = warp_tot[31];
  return v;
}

__global__ void __launch_bounds__(kBrickChunk) k_brick_sums(uint32_t* __restrict__ bt, int nb) {
  const int b = blockIdx.x * kBrickChunk + threadIdx.x;
  const uint4 v = b < nb ? reinterpret_cast<const uint4*>(bt)[b] : make_uint4(0u, 0u, 0u, 0u);
  uint4 tot;
  block_incl_scan4(v, &tot);
  if (threadIdx.x == 0) reinterpret_cast<uint4*>(bt)[nb + 1 + blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kBrickChunk) k_scan_bricks(uint32_t* __restrict__ bt, int nb) {
  // sums of the chunks before this one (at most kBrickChunk chunks)
  const int t = threadIdx.x;
  uint4 prev = t < (int)blockIdx.x ? reinterpret_cast<const uint4*>(bt)[nb + 1 + t] : make_uint4(0u, 0u, 0u, 0u);
  uint4 off;
  block_incl_scan4(prev, &off);
  __syncthreads();  // the scan's shared totals are reused below
  const int b = blockIdx.x * kBrickChunk + t;
  const uint4 v = b < nb ? reinterpret_cast<const uint4*>(bt)[b] : make_uint4(0u, 0u, 0u, 0u);
  uint4 tot;
  const uint4 incl = block_incl_scan4(v, &tot);
  const uint4 excl = make_uint4(incl.x - v.x, incl.y - v.y, incl.z - v.z, incl.w - v.w);
  if (b < nb) reinterpret_cast<uint4*>(bt)[b] = add4(off, excl);
  if (t == 0 && blockIdx.x == gridDim.x - 1) reinterpret_cast<uint4*>(bt)[nb] = add4(off, tot);
}

// Float expressions of findIntersection (MarchingCubesMesher.cu:98-100) with
// the corner point minC + idx * cellSize (MarchingCubesMesher.cu:1329-1331),
// evaluated with explicit rounding so that host and device agree bit for bit.
// The corner values are 0 or 1 and differ along an edge, so v2 - v1 is +1 or
// -1 and the IEEE quotient is the numerator or its negation, exactly
// (signed zeros included): no division is issued.
__device__ __forceinline__ float lerp_coord(float p1, float p2, float v1, float v2, float iso) {
  const float t = __fsub_rn(iso, v1);
  const float num = __fmul_rn(t, __fsub_rn(p2, p1));
  return __fadd_rn(p1, __fsub_rn(v2, v1) > 0.f ? num : -num);
}

__global__ void __launch_bounds__(kMcThreads, 6) k_mc_vertices(const uint8_t* __restrict__ C, GDims gd, McWin w,
                                                          const uint32_t* __restrict__ brick_off,
                                                          uint32_t* __restrict__ cell_voff,
                                                          float* __restrict__ V, float bx, float by, float bz,
                                                          float cs, float iso) {
  __shared__ __align__(16) uint8_t tile[kTileCells];
  __shared__ uint16_t list[kCellsPerBrick];
  int ox, oy, oz;
  brick_origin(blockIdx.x, ox, oy, oz);
  if (!brick_live(w, ox, oy, oz) || !load_tile_mixed(C, gd, ox, oy, oz, tile)) return;
  const int nc = brick_candidates(tile, w, ox, oy, oz, list);
  // the candidates in rounds of one per thread: a block scan of the round's
  // vertex counts gives each its first vertex, in list (Morton) order
  const uint32_t base = brick_off[4 * blockIdx.x + 1];
  uint32_t run = 0;
  for (int j0 = 0; j0 < nc; j0 += kMcThreads) {
    const int j = j0 + (int)threadIdx.x;
    int lx = 0, ly = 0, lz = 0, m = 0;
    int vals[8];
    uint32_t nvert = 0;
    if (j < nc) {
      local_coords(list[j], lx, ly, lz);
      cube_values(tile, lx, ly, lz, vals);
      m = mixed_mask(vals, true);
      if (m) nvert = cell_counts(vals, m).verts;
    }
    uint32_t round_total;
    const uint32_t pre = block_scan1(nvert, round_total);
    const uint32_t first = base + run + pre;
    run += round_total;
    if (!m) continue;
    const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
    uint32_t vo = first;
    cell_voff[gidx(gx, gy, gz, gd)] = vo;
    for (int s = 0; s < 8; s++) {
      if (!((m >> s) & 1)) continue;
      const int v = vals[s];
      const int em = edge_mask(v);
      // corner point from GLOBAL fine coordinates, so that a crop's vertices
      // are bit-identical to the whole grid's
      const int fx = 2 * (gx + w.off[0]) + (s & 1), fy = 2 * (gy + w.off[1]) + ((s >> 1) & 1),
                fz = 2 * (gz + w.off[2]) + (s >> 2);
      const float px = __fmaf_rn((float)fx, cs, bx);
      const float py = __fmaf_rn((float)fy, cs, by);
      const float pz = __fmaf_rn((float)fz, cs, bz);
      const float v0 = (v & 1) ? 1.f : 0.f, v1 = (v & 2) ? 1.f : 0.f, v3 = (v & 8) ? 1.f : 0.f,
                  v4 = (v & 16) ? 1.f : 0.f;
      if (em & 1) {  // edge 0: point -> point + (cs,0,0)
        float* o = V + 3 * (size_t)vo;
        o[0] = lerp_coord(px, __fadd_rn(px, cs), v0, v1, iso);
        o[1] = lerp_coord(py, py, v0, v1, iso);
        o[2] = lerp_coord(pz, pz, v0, v1, iso);
        vo++;
      }
      if (em & 8) {  // edge 3: point + (0,cs,0) -> point
        const float p1y = __fadd_rn(py, cs);
        float* o = V + 3 * (size_t)vo;
        o[0] = lerp_coord(px, px, v3, v0, iso);
        o[1] = lerp_coord(p1y, py, v3, v0, iso);
        o[2] = lerp_coord(pz, pz, v3, v0, iso);
        vo++;
      }
      if (em & 256) {  // edge 8: point -> point + (0,0,cs)
        float* o = V + 3 * (size_t)vo;
        o[0] = lerp_coord(px, px, v0, v4, iso);
        o[1] = lerp_coord(py, py, v0, v4, iso);
        o[2] = lerp_coord(pz, __fadd_rn(pz, cs), v0, v4, iso);
        vo++;
      }
    }
  }
}

// Per-cell summary used for neighbour lookups: bits 0..7 = mixed cubes,
// bits 8+k / 16+k / 24+k = cube k owns a vertex on edge 0 / 3 / 8.
__device__ __forceinline__ uint32_t cell_info(const uint8_t* tile, int lx, int ly, int lz, bool tagged) {
  if (!tagged || cell_uniform(tile, lx, ly, lz)) return 0u;
  int vals[8];
  cube_values(tile, lx, ly, lz, vals);
  const int m = mixed_mask(vals, true);
  uint32_t info = (uint32_t)m;
#pragma unroll
  for (int s = 0; s < 8; s++) {
    if (!((m >> s) & 1)) continue;
    const int em = edge_mask(vals[s]);
    info |= (uint32_t)(em & 1) << (8 + s);
    info |= (uint32_t)((em >> 3) & 1) << (16 + s);
    info |= (uint32_t)((em >> 8) & 1) << (24 + s);
  }
  return info;
}

constexpr int kInfoE = kBrick + 1;  // cells 0..16 of the brick (own + one neighbour layer)

__device__ __forceinline__ uint32_t info_of(const int vals[8], int m) {
  uint32_t info = (uint32_t)m;
#pragma unroll
  for (int s = 0; s < 8; s++) {
    if (!((m >> s) & 1)) continue;
    const int em = edge_mask(vals[s]);
    info |= (uint32_t)(em & 1) << (8 + s);
    info |= (uint32_t)((em >> 3) & 1) << (16 + s);
    info |= (uint32_t)((em >> 8) & 1) << (24 + s);
  }
  return info;
}

// dynamic shared memory of k_mc_triangles
constexpr size_t kTriSmem = sizeof(uint32_t) * kInfoE * kInfoE * kInfoE + sizeof(uint16_t) * kCellsPerBrick +
                            sizeof(uint16_t) * 8 * kMcThreads + kTileCells;

// Vertex offset of cube k of the cell whose summary is `info` (absent: -1),
// with its edge-0 / edge-3 ownership.
__device__ __forceinline__ long long cube_voff(uint32_t info, uint32_t cell_off, int k, int& e0, int& e3) {
  if (!((info >> k) & 1)) { e0 = e3 = 0; return -1; }
  const uint32_t below = info & ((1u << k) - 1u);
  const uint32_t off = cell_off + __popc((info >> 8) & below) + __popc((info >> 16) & below) +
                       __popc((info >> 24) & below);
  e0 = (info >> (8 + k)) & 1;
  e3 = (info >> (16 + k)) & 1;
  return (long long)off;
}

__global__ void __launch_bounds__(kMcThreads, 5) k_mc_triangles(const uint8_t* __restrict__ C, GDims gd, McWin w,
                                                              const uint32_t* __restrict__ brick_off,
                                                              const uint32_t* __restrict__ cell_voff,
                                                              uint32_t* __restrict__ T, uint32_t nt_total,
                                                              uint32_t* __restrict__ fix, int fix_cap) {
  extern __shared__ uint4 mc_smem[];
  uint8_t* tile = reinterpret_cast<uint8_t*>(mc_smem);                          // [18 * 18 rows of kTileP]
  uint32_t* info = reinterpret_cast<uint32_t*>(tile + kTileCells);              // [17^3]
  uint16_t* list = reinterpret_cast<uint16_t*>(info + kInfoE * kInfoE * kInfoE);  // [4096]
  int ox, oy, oz;
  brick_origin(blockIdx.x, ox, oy, oz);
  if (!brick_live(w, ox, oy, oz) || !load_tile_mixed(C, gd, ox, oy, oz, tile)) return;
  for (int i = threadIdx.x; i < kInfoE * kInfoE * kInfoE; i += blockDim.x) info[i] = 0u;
  const int nc = brick_candidates(tile, w, ox, oy, oz, list);
  // summaries of the own candidates
  for (int j = threadIdx.x; j < nc; j += blockDim.x) {
    int lx, ly, lz;
    local_coords(list[j], lx, ly, lz);
    int vals[8];
    cube_values(tile, lx, ly, lz, vals);
    info[lx + kInfoE * (ly + kInfoE * lz)] = info_of(vals, mixed_mask(vals, true));
  }
  // the neighbour layer (cells 16 along some axis)
  for (int i = threadIdx.x; i < kInfoE * kInfoE * kInfoE; i += blockDim.x) {
    const int lx = i % kInfoE, ly = (i / kInfoE) % kInfoE, lz = i / (kInfoE * kInfoE);
    if (lx < kBrick && ly < kBrick && lz < kBrick) continue;
    info[i] = cell_info(tile, lx, ly, lz, win_tag(w, ox + lx, oy + ly, oz + lz));
  }
  __syncthreads();
  // The candidates in rounds of one per thread; each round's mixed cubes
  // (cell in list order, then sub-cube order) go to a cube list and are
  // worked one per thread, a block scan of their triangle counts giving
  // each its first triangle: the order of the cell-by-cell walk, without
  // the lanes of a warp waiting on each other's sub-cube loops.
  uint16_t* cubes = list + kCellsPerBrick;  // [8 * kMcThreads]: (cell slot << 3) | sub-cube
  const uint32_t tbase = brick_off[4 * blockIdx.x + 2];
  uint32_t run = 0;
  for (int j0 = 0; j0 < nc; j0 += kMcThreads) {
    const int j = j0 + (int)threadIdx.x;
    uint32_t m = 0;
    if (j < nc) {
      int lx, ly, lz;
      local_coords(list[j], lx, ly, lz);
      m = info[lx + kInfoE * (ly + kInfoE * lz)] & 0xffu;
      if (m != 0 && !win_emit(w, ox + lx, oy + ly, oz + lz)) m = 0;
    }
    uint32_t nround;
    uint32_t k = block_scan1((uint32_t)__popc(m), nround);
    while (m) {
      const int sc = __ffs(m) - 1;
      m &= m - 1;
      cubes[k++] = (uint16_t)((threadIdx.x << 3) | sc);
    }
    __syncthreads();
    for (int c0 = 0; c0 < (int)nround; c0 += kMcThreads) {
      const int c = c0 + (int)threadIdx.x;
      int lx = 0, ly = 0, lz = 0, s = 0, v = 0, cnt = 0;
      if (c < (int)nround) {
        const int e = cubes[c];
        s = e & 7;
        local_coords(list[j0 + (e >> 3)], lx, ly, lz);
        v = cube_value(tile, lx, ly, lz, s);
        cnt = c_tri_count[v];
      }
      uint32_t ttot;
      const uint32_t pre = block_scan1((uint32_t)cnt, ttot);
      const uint32_t to = tbase + run + pre;
      run += ttot;
      if (c >= (int)nround) continue;
      const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
      const int em = edge_mask(v);
      const int fx = 2 * gx + (s & 1), fy = 2 * gy + ((s >> 1) & 1), fz = 2 * gz + (s >> 2);  // local
      int o0 = 0, o3 = 0;
      const uint32_t vo = (uint32_t)cube_voff(info[lx + kInfoE * (ly + kInfoE * lz)],
                                              cell_voff[gidx(gx, gy, gz, gd)], s, o0, o3);
      uint32_t vert[12];
#pragma unroll
      for (int e = 0; e < 12; e++) vert[e] = 0;
      {
        uint32_t ind = 0;
        if (em & 1) vert[0] = vo + ind++;
        if (em & 8) vert[3] = vo + ind++;
        if (em & 256) vert[8] = vo + ind++;
      }
      // neighbour cubes +x, +x+y, +y, +z, +x+z, +y+z (BuildNeighbors order,
      // GMorpho.cu:6480-6487) and the edges they own
      // (MarchingCubesMesher.cu:1392-1456)
      auto nb = [&](int dx, int dy, int dz, int& e0, int& e3) -> long long {
        const int nfx = fx + dx, nfy = fy + dy, nfz = fz + dz;
        const int cx = (nfx >> 1) - ox, cy = (nfy >> 1) - oy, cz = (nfz >> 1) - oz;
        const uint32_t ninfo = info[cx + kInfoE * (cy + kInfoE * cz)];
        const int kk = (nfx & 1) | ((nfy & 1) << 1) | ((nfz & 1) << 2);
        if (!((ninfo >> kk) & 1)) { e0 = e3 = 0; return -1; }
        return cube_voff(ninfo, cell_voff[gidx(nfx >> 1, nfy >> 1, nfz >> 1, gd)], kk, e0, e3);
      };
      int a0 = 0, a3 = 0;
      if (em & (2 | 512)) {
        const long long id1 = nb(1, 0, 0, a0, a3);
        if ((em & 2) && id1 >= 0) vert[1] = (uint32_t)id1 + a0;
        if (em & 512) vert[9] = id1 >= 0 ? (uint32_t)id1 + a0 + a3 : 0u;
      }
      if (em & 1024) {
        const long long id2 = nb(1, 1, 0, a0, a3);
        vert[10] = id2 >= 0 ? (uint32_t)id2 + a0 + a3 : 0u;
      }
      if (em & (4 | 2048)) {
        const long long id3 = nb(0, 1, 0, a0, a3);
        if (em & 4) vert[2] = id3 >= 0 ? (uint32_t)id3 : 0u;
        if (em & 2048) vert[11] = id3 >= 0 ? (uint32_t)id3 + a0 + a3 : 0u;
      }
      if (em & (16 | 128)) {
        const long long id4 = nb(0, 0, 1, a0, a3);
        if (em & 16) vert[4] = id4 >= 0 ? (uint32_t)id4 : 0u;
        if ((em & 128) && id4 >= 0) vert[7] = (uint32_t)id4 + a0;
      }
      if (em & 32) {
        const long long id5 = nb(1, 0, 1, a0, a3);
        if (id5 >= 0) vert[5] = (uint32_t)id5 + a0;
      }
      if (em & 64) {
        const long long id7 = nb(0, 1, 1, a0, a3);
        vert[6] = id7 >= 0 ? (uint32_t)id7 : 0u;
      }
      // reversed winding (MarchingCubesMesher.cu:1487-1497)
      const uint64_t tl = c_tri_packed[v];
      for (int t = 0; t < cnt; t++) {
        uint32_t* o = T + 3 * (size_t)(to + t);
        o[0] = vert[(tl >> (4 * (3 * t + 2))) & 0xf];
        o[1] = vert[(tl >> (4 * (3 * t + 1))) & 0xf];
        o[2] = vert[(tl >> (4 * (3 * t))) & 0xf];
      }
      if (c_tri_len[v] > cnt) {
        // Case 91: the reference writes one more triangle than its slot
        // count; it lands on the next slot (the next cube's first triangle)
        // and, written later, wins; past the end it is dropped.
        const uint32_t slot = to + cnt;
        if (slot < nt_total) {
          const int idx = (int)atomicAdd(fix, 1u);
          if (idx < fix_cap) {
            uint32_t* f = fix + 1 + 4 * idx;
            f[0] = slot;
            f[1] = vert[(tl >> (4 * (3 * cnt + 2))) & 0xf];
            f[2] = vert[(tl >> (4 * (3 * cnt + 1))) & 0xf];
            f[3] = vert[(tl >> (4 * (3 * cnt))) & 0xf];
          }
        }
      }
    }
    __syncthreads();  // the cube list is rewritten by the next round
  }
}

__global__ void k_mc_fix91(const uint32_t* __restrict__ fix, int fix_cap, uint32_t* __restrict__ T) {
  const int n = min((int)fix[0], fix_cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t* f = fix + 1 + 4 * i;
    uint32_t* o = T + 3 * (size_t)f[0];
    o[0] = f[1]; o[1] = f[2]; o[2] = f[3];
  }
}

// ------------------------------------------------------------------ normals

// Vertex -> corner lists.  Corners of a vertex are listed in corner order
// (the reference's per-vertex accumulation order).  Vertex 0 is special: the
// reference's triangles take index 0 for an edge whose owning cube is not
// tagged (cubes of border cells), so on grids whose surface reaches the
// border vertex 0 collects an unbounded number of corners.  Its row is
// built by an order-preserving compaction over all corners (linear), the
// other rows (at most 20 corners each) by atomics and an in-row sort.
__global__ void k_adj_count(const uint32_t* __restrict__ T, int64_t nt, uint32_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 3 * nt; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t v = T[i];
    if (v != 0u) atomicAdd(cnt + v, 1u);
  }
}

constexpr int kRow0Chunk = 2048;  // corners per block (256 threads x 8)

// corners of vertex 0 per chunk of kRow0Chunk corners
__global__ void __launch_bounds__(256) k_row0_count(const uint32_t* __restrict__ T, int64_t n,
                                                     uint32_t* __restrict__ counts) {
  __shared__ uint32_t ws[8];
  const int64_t base = (int64_t)blockIdx.x * kRow0Chunk;
  uint32_t c = 0;
  for (int i = threadIdx.x; i < kRow0Chunk; i += 256)
    if (base + i < n) c += T[base + i] == 0u;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < 8; w++) t += ws[w];
    counts[blockIdx.x] = t;
  }
}

// the count of vertex 0 (total of the scanned chunk counts) into cnt[0]
__global__ void k_row0_total(const uint32_t* __restrict__ offs, int nchunks, uint32_t* __restrict__ cnt) {
  if (threadIdx.x == 0 && blockIdx.x == 0) cnt[0] = offs[nchunks];
}

// row 0 in corner order: chunk offset + rank inside the chunk
__global__ void __launch_bounds__(256) k_row0_fill(const uint32_t* __restrict__ T, int64_t n,
                                                    const uint32_t* __restrict__ offs,
                                                    const uint32_t* __restrict__ rowptr, uint32_t* __restrict__ adj) {
  __shared__ uint32_t wtot[8];
  const int64_t base = (int64_t)blockIdx.x * kRow0Chunk + (int64_t)threadIdx.x * 8;
  uint32_t f = 0, s = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const bool z = base + j < n && T[base + j] == 0u;
    f |= (z ? 1u : 0u) << j;
    s += z ? 1u : 0u;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) wtot[wid] = x;
  __syncthreads();
  uint32_t pos = rowptr[0] + offs[blockIdx.x] + x - s;
  for (int w = 0; w < wid; w++) pos += wtot[w];
#pragma unroll
  for (int j = 0; j < 8; j++)
    if ((f >> j) & 1u) adj[pos++] = (uint32_t)(base + j);
}

// Exclusive scan of n u32 into out[0..n] in three kernels: per-block sums of
// 2048-element chunks, a scan of the block sums, then per-chunk scans.
constexpr int kScanChunk = 2048;

__global__ void __launch_bounds__(256) k_scan_sums(const uint32_t* __restrict__ in, int64_t n,
                                                    uint32_t* __restrict__ sums) {
  __shared__ uint32_t ws[8];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk;
  uint32_t s = 0;
  for (int i = threadIdx.x; i < kScanChunk; i += 256)
    if (base + i < n) s += in[base + i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < 8; w++) t += ws[w];
    sums[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(1024) k_scan_small(uint32_t* __restrict__ v, int n) {
  __shared__ uint32_t part[1024];
  const int t = threadIdx.x;
  const int per = (n + 1023) / 1024;
  const int b0 = t * per, b1 = min(n, b0 + per);
  uint32_t s = 0;
  for (int b = b0; b < b1; b++) s += v[b];
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const uint32_t x = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += x;
    __syncthreads();
  }
  uint32_t run = part[t] - s;
  for (int b = b0; b < b1; b++) {
    const uint32_t x = v[b];
    v[b] = run;
    run += x;
  }
  if (t == 1023) v[n] = part[1023];
}

__global__ void __launch_bounds__(256) k_scan_apply(const uint32_t* __restrict__ in, int64_t n,
                                                     const uint32_t* __restrict__ sums, uint32_t* __restrict__ out) {
  __shared__ uint32_t wtot[8];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * 8;
  uint32_t v[8], s = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    v[j] = base + j < n ? in[base + j] : 0u;
    s += v[j];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) wtot[wid] = x;
  __syncthreads();
  uint32_t wpre = 0;
  for (int w = 0; w < wid; w++) wpre += wtot[w];
  uint32_t run = sums[blockIdx.x] + wpre + x - s;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 255) out[n] = sums[gridDim.x];
}

__global__ void k_adj_fill(const uint32_t* __restrict__ T, int64_t nt, const uint32_t* __restrict__ rowptr,
                           uint32_t* __restrict__ cursor, uint32_t* __restrict__ adj) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 3 * nt; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t v = T[i];
    if (v == 0u) continue;  // row 0: k_row0_fill
    const uint32_t slot = atomicAdd(cursor + v, 1u);
    adj[rowptr[v] + slot] = (uint32_t)i;  // corner id = 3 t + role
  }
}


__device__ __forceinline__ float3 ld3(const float* p, uint32_t i) {
  return make_float3(p[3 * (size_t)i], p[3 * (size_t)i + 1], p[3 * (size_t)i + 2]);
}

__device__ __forceinline__ float3 normalize3(float3 n) {
  const float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(n.x, n.x), __fmul_rn(n.y, n.y)), __fmul_rn(n.z, n.z)));
  return make_float3(__fdiv_rn(n.x, l), __fdiv_rn(n.y, l), __fdiv_rn(n.z, l));
}


__device__ __forceinline__ float dist2(float3 a, float3 b) {
  const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}


__device__ __forceinline__ float dist2n(float4 a, float4 b) {
  const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// The per-vertex steps after the incident-triangle lists are filled, in
// one kernel: the list sorted into triangle order (in registers, a bitonic
// network over 8 or 16 slots; vertex 0's row is already in order, longer
// lists are sorted in place); the area-weighted normal (ComputeMeshNormals,
// GMorpho.cu:6498-6524) summed in that order and normalised
// (GMorpho.cu:6526-6537); and, when the normals are filtered, each corner's
// filter record: the other two vertices b, c in the reference's order and
// the iteration-invariant position terms |pa - pb|^2 / sigma_p^2
// (GMorpho.cu:6561-6569) — sigma_p is 1 (GMorpho.cu:6959-6969), so the term
// is the squared distance itself (an IEEE division by 1 is exact).  Every
// incident triangle's vertices and positions are loaded once for both.
template <int M>
__device__ __forceinline__ void bitonic_sort(uint32_t (&k)[M]) {
#pragma unroll
  for (int s = 2; s <= M; s <<= 1)
#pragma unroll
    for (int j = s >> 1; j > 0; j >>= 1)
#pragma unroll
      for (int i = 0; i < M; i++) {
        const int l = i ^ j;
        if (l > i) {
          const uint32_t a = k[i], b = k[l];
          const bool up = (i & s) == 0;
          k[i] = up ? min(a, b) : max(a, b);
          k[l] = up ? max(a, b) : min(a, b);
        }
      }
}

// one incident corner: its triangle's normal term, and its filter record
__device__ __forceinline__ void adj_corner(const float* __restrict__ V, const uint32_t* __restrict__ T,
                                           uint32_t corner, const float3& pa, float3& acc, uint64_t* pair) {
  const uint32_t t = corner / 3, role = corner - 3 * t;
  const uint32_t i0 = T[3 * (size_t)t], i1 = T[3 * (size_t)t + 1], i2 = T[3 * (size_t)t + 2];
  const float3 p0 = ld3(V, i0), p1 = ld3(V, i1), p2 = ld3(V, i2);
  const float3 a = make_float3(__fsub_rn(p1.x, p0.x), __fsub_rn(p1.y, p0.y), __fsub_rn(p1.z, p0.z));
  const float3 b = make_float3(__fsub_rn(p2.x, p0.x), __fsub_rn(p2.y, p0.y), __fsub_rn(p2.z, p0.z));
  const float nx = __fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y));
  const float ny = __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z));
  const float nz = __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x));
  acc = make_float3(__fadd_rn(acc.x, nx), __fadd_rn(acc.y, ny), __fadd_rn(acc.z, nz));
  if (pair) {
    // the other two vertices (reference order (1, 2), (0, 2), (0, 1)) as
    // (vertex << 32 | position term bits)
    const uint32_t ib = role == 0 ? i1 : i0, ic = role == 2 ? i1 : i2;
    const float3 pb = role == 0 ? p1 : p0, pc = role == 2 ? p1 : p2;
    pair[0] = ((uint64_t)ib << 32) | __float_as_uint(dist2(pa, pb));
    pair[1] = ((uint64_t)ic << 32) | __float_as_uint(dist2(pa, pc));
  }
}

template <int M>
__device__ __forceinline__ void bitonic_sort64(uint64_t (&k)[M]) {
#pragma unroll
  for (int s = 2; s <= M; s <<= 1)
#pragma unroll
    for (int j = s >> 1; j > 0; j >>= 1)
#pragma unroll
      for (int i = 0; i < M; i++) {
        const int l = i ^ j;
        if (l > i) {
          const uint64_t a = k[i], b = k[l];
          const bool up = (i & s) == 0;
          k[i] = up ? (a < b ? a : b) : (a < b ? b : a);
          k[l] = up ? (a < b ? b : a) : (a < b ? a : b);
        }
      }
}

// The filter records of a vertex from its neighbour pairs sorted by
// (vertex, term): one record per neighbour, or per two occurrences of it
// (an edge shared by two incident triangles), the sign bit marking a
// double.  Returns the number of records written.
__device__ __forceinline__ uint32_t put_records(const uint64_t* kv, int m, uint2* rec) {
  uint32_t w = 0;
  int run = 0;
  for (int i = 0; i < m; i++) {
    if (kv[i] == ~0ull) break;
    run = (i > 0 && (kv[i] >> 32) == (kv[i - 1] >> 32)) ? run + 1 : 0;
    if (run & 1) continue;
    const bool dbl = i + 1 < m && kv[i + 1] != ~0ull && (kv[i + 1] >> 32) == (kv[i] >> 32);
    rec[w++] = make_uint2((uint32_t)(kv[i] >> 32), (uint32_t)kv[i] | (dbl ? 0x80000000u : 0u));
  }
  return w;
}

__global__ void __launch_bounds__(256, 4) k_adj_finish(const float* __restrict__ V, const uint32_t* __restrict__ T,
                             const uint32_t* __restrict__ rowptr, uint32_t* __restrict__ adj, int64_t nv,
                             int zero_isolated, float4* __restrict__ N4, float* __restrict__ N3,
                             uint2* __restrict__ ent, uint32_t* __restrict__ ncnt) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t b = rowptr[v], e = rowptr[v + 1], n = e - b;
    if (zero_isolated && n == 0) {
      N4[v] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (N3) { N3[3 * v] = 0.f; N3[3 * v + 1] = 0.f; N3[3 * v + 2] = 0.f; }
      if (ent) ncnt[v] = 0;
      continue;
    }
    const float3 pa = ld3(V, (uint32_t)v);
    float3 acc = make_float3(0.f, 0.f, 0.f);
    if (v != 0 && n <= 8) {
      uint32_t key[8];
      uint64_t kv[16];
#pragma unroll
      for (int k = 0; k < 8; k++) key[k] = (uint32_t)k < n ? adj[b + k] : 0xffffffffu;
      bitonic_sort<8>(key);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        kv[2 * k] = kv[2 * k + 1] = ~0ull;
        if ((uint32_t)k < n) {
          adj[b + k] = key[k];
          adj_corner(V, T, key[k], pa, acc, ent ? kv + 2 * k : nullptr);
        }
      }
      if (ent) {
        bitonic_sort64<16>(kv);
        ncnt[v] = put_records(kv, 16, ent + 2 * (size_t)b);
      }
    } else {
      // rare (more than 8 incident triangles): sorted in memory
      if (v != 0)
        for (uint32_t i = b + 1; i < e; i++) {  // in place (vertex 0's row is already in order)
          const uint32_t key = adj[i];
          uint32_t j = i;
          while (j > b && adj[j - 1] > key) { adj[j] = adj[j - 1]; j--; }
          adj[j] = key;
        }
      // the pairs in the record slots, sorted there, then merged in place
      uint64_t* kv = ent ? reinterpret_cast<uint64_t*>(ent + 2 * (size_t)b) : nullptr;
      for (uint32_t i = b; i < e; i++) adj_corner(V, T, adj[i], pa, acc, kv ? kv + 2 * (i - b) : nullptr);
      if (kv) {
        const uint32_t m = 2 * n;
        for (uint32_t i = 1; i < m; i++) {
          const uint64_t x = kv[i];
          uint32_t j = i;
          while (j > 0 && kv[j - 1] > x) { kv[j] = kv[j - 1]; j--; }
          kv[j] = x;
        }
        // merged records never overtake the pairs still to be read
        uint32_t w = 0;
        int run = 0;
        uint32_t prev = 0;
        for (uint32_t i = 0; i < m; i++) {
          const uint64_t x = kv[i];
          const uint32_t id = (uint32_t)(x >> 32);
          run = (i > 0 && id == prev) ? run + 1 : 0;
          prev = id;
          if (run & 1) continue;
          const bool dbl = i + 1 < m && (uint32_t)(kv[i + 1] >> 32) == id;
          ent[2 * (size_t)b + w++] = make_uint2(id, (uint32_t)x | (dbl ? 0x80000000u : 0u));
        }
        ncnt[v] = w;
      }
    }
    const float3 nn = normalize3(acc);
    N4[v] = make_float4(nn.x, nn.y, nn.z, 0.f);
    if (N3) { N3[3 * v] = nn.x; N3[3 * v + 1] = nn.y; N3[3 * v + 2] = nn.z; }
  }
}

// Packs each vertex's records (built from 2 rowptr[v], roff from the scan
// of their counts) so that the iterations read them contiguously.
__global__ void k_rec_pack(const uint2* __restrict__ ent, const uint32_t* __restrict__ rowptr,
                           const uint32_t* __restrict__ roff, int64_t nv, uint2* __restrict__ rec) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const uint2* src = ent + 2 * (size_t)rowptr[v];
    const uint32_t r0 = roff[v], n = roff[v + 1] - r0;
    for (uint32_t i = 0; i < n; i++) rec[r0 + i] = src[i];
  }
}

// One bilateral normal iteration (BilateralMeshFiltering{,Normalize},
// GMorpho.cu:6539-6620): each incident triangle adds w1 n_b + w2 n_c.  A
// neighbour shared by two incident triangles appears twice in that sum with
// the same weight; its record (8 bytes: vertex, position term) carries the
// doubling in the sign bit, so that each neighbour is read once.  The sum
// runs over the neighbours in vertex order (deterministic).
// one neighbour's term, added to acc
__device__ __forceinline__ void bilateral_add(float3& acc, uint2 e, float4 nb, float4 na, float sn2) {
  // the reference library is built with -use_fast_math (GMorpho/cuda.prf:47),
  // so its exp and division here are the fast forms
  float w = __expf(-__fadd_rn(__uint_as_float(e.y & 0x7fffffffu), __fdividef(dist2n(na, nb), sn2)));
  if (e.y >> 31) w = __fadd_rn(w, w);
  acc.x = __fadd_rn(acc.x, __fmul_rn(w, nb.x));
  acc.y = __fadd_rn(acc.y, __fmul_rn(w, nb.y));
  acc.z = __fadd_rn(acc.z, __fmul_rn(w, nb.z));
}

// The records two at a time, the next two loaded one step ahead, so that
// two neighbour-normal gathers are in flight per thread; the terms are
// added in record order (the same sum, bit for bit, as one at a time).
__device__ __forceinline__ float3 bilateral_sum(const float4* __restrict__ Nin, const uint2* __restrict__ rec,
                                                uint32_t n, float4 na, float sn2) {
  float3 acc = make_float3(0.f, 0.f, 0.f);
  const uint2 z2 = make_uint2(0u, 0u);
  uint2 f0 = n > 0 ? rec[0] : z2, f1 = n > 1 ? rec[1] : z2;  // the next pair
  uint32_t i = 0;
  for (; i + 1 < n; i += 2) {
    const uint2 e0 = f0, e1 = f1;
    if (i + 2 < n) f0 = rec[i + 2];
    if (i + 3 < n) f1 = rec[i + 3];
    const float4 nb0 = Nin[e0.x], nb1 = Nin[e1.x];
    bilateral_add(acc, e0, nb0, na, sn2);
    bilateral_add(acc, e1, nb1, na, sn2);
  }
  if (i < n) bilateral_add(acc, f0, Nin[f0.x], na, sn2);
  return acc;
}

__global__ void k_bilateral(const float4* __restrict__ Nin, const uint32_t* __restrict__ roff,
                            const uint2* __restrict__ rec, int64_t nv, float sn2, int zero_isolated,
                            float4* __restrict__ Nout, float* __restrict__ N3) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t r0 = roff[v], n = roff[v + 1] - r0;
    if (zero_isolated && n == 0) {
      Nout[v] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (N3) { N3[3 * v] = 0.f; N3[3 * v + 1] = 0.f; N3[3 * v + 2] = 0.f; }
      continue;
    }
    const float3 acc = bilateral_sum(Nin, rec + r0, n, Nin[v], sn2);
    const float3 nn = normalize3(acc);
    Nout[v] = make_float4(nn.x, nn.y, nn.z, 0.f);
    if (N3) { N3[3 * v] = nn.x; N3[3 * v + 1] = nn.y; N3[3 * v + 2] = nn.z; }
  }
}

// The same iteration over the vertices of several meshes at once (one
// launch per iteration for a batch): vertex g of the concatenation belongs
// to the mesh m with start[m] <= g < start[m + 1].
struct BilMesh {
  const float4* Na;       // normals of even iterations' inputs (N4a)
  float4* Nb;             // and odd (N4b)
  const uint32_t* roff;
  const uint2* rec;
  float* N3;              // final normals (last iteration)
  int zero_isolated;
};

__global__ void k_bilateral_group(const BilMesh* __restrict__ meshes, const int64_t* __restrict__ start, int n,
                                  int odd, int last, float sn2) {
  const int64_t total = start[n];
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = n - 1;  // last m with start[m] <= g
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (start[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const BilMesh& M = meshes[lo];
    const int64_t v = g - start[lo];
    const float4* Nin = odd ? M.Nb : M.Na;
    float4* Nout = odd ? const_cast<float4*>(M.Na) : M.Nb;
    float* N3 = last ? M.N3 : nullptr;
    const uint32_t r0 = M.roff[v], nrec = M.roff[v + 1] - r0;
    if (M.zero_isolated && nrec == 0) {
      Nout[v] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (N3) { N3[3 * v] = 0.f; N3[3 * v + 1] = 0.f; N3[3 * v + 2] = 0.f; }
      continue;
    }
    const float3 acc = bilateral_sum(Nin, M.rec + r0, nrec, Nin[v], sn2);
    const float3 nn = normalize3(acc);
    Nout[v] = make_float4(nn.x, nn.y, nn.z, 0.f);
    if (N3) { N3[3 * v] = nn.x; N3[3 * v + 1] = nn.y; N3[3 * v + 2] = nn.z; }
  }
}

// ------------------------------------------------------------------ host

static int gs_blocks(int64_t n, int threads, int sms) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)(sms > 0 ? sms : 152) * 16;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

// Grid of a grid-stride kernel as one wave of resident blocks (SMs x the
// blocks of 256 threads one SM holds at once), at most one block per 256
// items: the filter iterations measured 8% faster so than with two waves.
static int wave_blocks(const void* kernel, int64_t n, int sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  int64_t b = (int64_t)(sms > 0 ? sms : 152) * per_sm;
  const int64_t need = (n + 255) / 256;
  if (b > need) b = need;
  return (int)(b < 1 ? 1 : b);
}

void MeshBuffers::release() {
  cudaFree(V); cudaFree(N); cudaFree(N2); cudaFree(N4a); cudaFree(N4b); cudaFree(T); cudaFree(adj);
  cudaFree(ent); cudaFree(rec); cudaFree(roff); cudaFree(rowptr); cudaFree(cursor); cudaFree(cell_voff); cudaFree(brick_tot);
  cudaFree(fix);
  *this = MeshBuffers();
}

// Bricks are visited in Morton order over the smallest power-of-two cube of
// bricks covering the grid; bricks outside the grid or the tag box return
// at once.
static int brick_count(const int d[3]) {
  const int m = d[0] > d[1] ? (d[0] > d[2] ? d[0] : d[2]) : (d[1] > d[2] ? d[1] : d[2]);
  int p = kBrick;
  while (p < m) p *= 2;
  const int e = p / kBrick;
  return e * e * e;
}

static void grid_dims(const MeshArgs& a, int d[3]) {
  for (int k = 0; k < 3; k++) d[k] = a.dims[0] > 0 ? a.dims[k] : a.res;
}

static McWin window_of(const MeshArgs& a) {
  McWin w;
  int d[3];
  grid_dims(a, d);
  const bool crop = a.gres > 0;
  for (int k = 0; k < 3; k++) {
    w.gdim[k] = crop ? a.gres : d[k];
    w.off[k] = crop ? a.off[k] : 0;
    w.tlo[k] = crop ? a.tag_lo[k] : 0;
    w.thi[k] = crop ? a.tag_hi[k] : d[k];
    w.elo[k] = crop ? a.emit_lo[k] : 0;
    w.ehi[k] = crop ? a.emit_hi[k] : d[k];
  }
  return w;
}

// capacity helpers: buffers grow (never shrink) to the sizes asked for
static cudaError_t ensure_grid_buffers(MeshBuffers& b, int64_t cells, int nb) {
  cudaError_t e;
  if (nb + 1 > b.bricks_cap) {
    if (b.brick_tot) cudaFree(b.brick_tot);
    b.brick_tot = nullptr;
    // counters and totals (nb + 1), then the chunk sums of the scan
    e = cudaMalloc(&b.brick_tot, sizeof(uint32_t) * 4 * ((size_t)nb + 1 + (nb + kBrickChunk - 1) / kBrickChunk));
    if (e != cudaSuccess) return e;
    b.bricks_cap = nb + 1;
  }
  if (cells > b.cells_cap) {
    if (b.cell_voff) cudaFree(b.cell_voff);
    b.cell_voff = nullptr;
    e = cudaMalloc(&b.cell_voff, sizeof(uint32_t) * (size_t)cells);
    if (e != cudaSuccess) return e;
    b.cells_cap = cells;
  }
  return cudaSuccess;
}

static cudaError_t ensure_vertex_buffers(MeshBuffers& b, int64_t nv) {
  cudaError_t e;
  if (b.v_cap < nv || b.V == nullptr) {
    cudaFree(b.V); cudaFree(b.N); cudaFree(b.N4a); cudaFree(b.N4b); cudaFree(b.rowptr); cudaFree(b.cursor);
    cudaFree(b.roff);
    b.V = b.N = nullptr;
    b.N4a = b.N4b = nullptr;
    b.rowptr = b.cursor = nullptr;
    b.roff = nullptr;
    b.v_cap = 0;
    const int64_t c = nv + nv / 4 + 1024;
    if ((e = cudaMalloc(&b.V, sizeof(float) * 3 * (size_t)c)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&b.N, sizeof(float) * 3 * (size_t)c)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&b.N4a, sizeof(float4) * (size_t)c)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&b.N4b, sizeof(float4) * (size_t)c)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&b.rowptr, sizeof(uint32_t) * ((size_t)c + 1))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&b.cursor, sizeof(uint32_t) * ((size_t)c + 1))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&b.roff, sizeof(uint32_t) * ((size_t)c + 1))) != cudaSuccess) return e;
    b.v_cap = c;
  }
  return cudaSuccess;
}

static cudaError_t ensure_triangle_buffers(MeshBuffers& b, int64_t nt) {
  cudaError_t e;
  if (b.t_cap < nt || b.T == nullptr) {
    cudaFree(b.T); cudaFree(b.adj); cudaFree(b.ent); cudaFree(b.rec);
    b.T = b.adj = nullptr;
    b.ent = b.rec = nullptr;
    b.t_cap = 0;
    const int64_t c = nt + nt / 4 + 1024;
    if ((e = cudaMalloc(&b.T, sizeof(uint32_t) * 3 * (size_t)c)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&b.adj, sizeof(uint32_t) * 3 * (size_t)c)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&b.ent, sizeof(uint2) * 6 * (size_t)c)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&b.rec, sizeof(uint2) * 6 * (size_t)c)) != cudaSuccess) return e;
    b.t_cap = c;
  }
  return cudaSuccess;
}

cudaError_t mesh_reserve(MeshBuffers& b, int res, int64_t nv, int64_t nt) {
  const int d[3] = {res, res, res};
  cudaError_t e = ensure_grid_buffers(b, (int64_t)res * res * res, brick_count(d));
  if (e == cudaSuccess) e = ensure_vertex_buffers(b, nv);
  if (e == cudaSuccess) e = ensure_triangle_buffers(b, nt);
  return e;
}

cudaError_t mesh_count_launch(const MeshArgs& a, MeshBuffers& b, cudaStream_t st, KernelCounter* kc,
                              uint32_t* h_tot4) {
  int d[3];
  grid_dims(a, d);
  const GDims gd{d[0], d[1], d[2]};
  const int64_t cells = (int64_t)d[0] * d[1] * d[2];
  const int nb = brick_count(d);
  cudaError_t e = ensure_grid_buffers(b, cells, nb);
  if (e != cudaSuccess) return e;
  GM_LAUNCH(kc, "k_mc_count", st, k_mc_count<<<nb, kMcThreads, 0, st>>>(a.C, gd, window_of(a), b.brick_tot));
  {
    const int nchunks = (nb + kBrickChunk - 1) / kBrickChunk;
    if (nchunks > kBrickChunk) return cudaErrorInvalidValue;
    GM_LAUNCH(kc, "k_brick_sums", st, k_brick_sums<<<nchunks, kBrickChunk, 0, st>>>(b.brick_tot, nb));
    GM_LAUNCH(kc, "k_scan_bricks", st, k_scan_bricks<<<nchunks, kBrickChunk, 0, st>>>(b.brick_tot, nb));
  }
  return cudaMemcpyAsync(h_tot4, b.brick_tot + 4 * (size_t)nb, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
}

cudaError_t mesh_prepare_grid(const MeshArgs& a, MeshBuffers& b) {
  int d[3];
  grid_dims(a, d);
  return ensure_grid_buffers(b, (int64_t)d[0] * d[1] * d[2], brick_count(d));
}

cudaError_t mesh_count_finish(MeshBuffers& b, const uint32_t* tot, int64_t* nv, int64_t* nt) {
  *nv = tot[1];
  *nt = tot[2];
  const int need_fix = (int)tot[3];
  if (need_fix + 1 > b.fix_cap || b.fix == nullptr) {
    if (b.fix) cudaFree(b.fix);
    b.fix = nullptr;
    const int c = need_fix + 64;
    cudaError_t e = cudaMalloc(&b.fix, sizeof(uint32_t) * (1 + 4 * (size_t)c));
    if (e != cudaSuccess) return e;
    b.fix_cap = c;
  }
  return cudaSuccess;
}

cudaError_t mesh_count(const MeshArgs& a, MeshBuffers& b, cudaStream_t st, KernelCounter* kc, int64_t* nv,
                       int64_t* nt) {
  uint32_t tot[4];
  cudaError_t e = mesh_count_launch(a, b, st, kc, tot);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  e = mesh_count_finish(b, tot, nv, nt);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t mesh_emit(const MeshArgs& a, MeshBuffers& b, int64_t nv, int64_t nt, cudaStream_t st,
                      KernelCounter* kc) {
  int d[3];
  grid_dims(a, d);
  const GDims gd{d[0], d[1], d[2]};
  const int nb = brick_count(d);
  const McWin w = window_of(a);
  cudaError_t e;
  // per-vertex buffers share one capacity, per-triangle buffers another
  if ((e = ensure_vertex_buffers(b, nv)) != cudaSuccess) return e;
  if ((e = ensure_triangle_buffers(b, nt)) != cudaSuccess) return e;
  const float cs = 0.5f * a.cell_size;  // exact: scaling by a power of two
  cudaMemsetAsync(b.fix, 0, sizeof(uint32_t), st);
  GM_LAUNCH(kc, "k_mc_vertices", st, k_mc_vertices<<<nb, kMcThreads, 0, st>>>(a.C, gd, w, b.brick_tot, b.cell_voff, b.V, a.bbox_min[0], a.bbox_min[1],
                                           a.bbox_min[2], cs, a.isovalue));
  ensure_dynamic_smem(reinterpret_cast<const void*>(k_mc_triangles), kTriSmem);
  GM_LAUNCH(kc, "k_mc_triangles", st, k_mc_triangles<<<nb, kMcThreads, kTriSmem, st>>>(a.C, gd, w, b.brick_tot, b.cell_voff, b.T, (uint32_t)nt, b.fix,
                                            b.fix_cap));
  GM_LAUNCH(kc, "k_mc_fix91", st, k_mc_fix91<<<1, 256, 0, st>>>(b.fix, b.fix_cap, b.T));
  if (a.geometry_done) cudaEventRecord(a.geometry_done, st);
  if (nv == 0 || nt == 0) return cudaGetLastError();
  // normals
  const int sms = a.num_sms;
  const int nchunks = (int)((nv + kScanChunk - 1) / kScanChunk);
  const int nchunks0 = (int)((3 * nt + kRow0Chunk - 1) / kRow0Chunk);
  // chunk sums (rows, then row 0) go to the per-cell offsets buffer, unused
  // once the triangles are out
  if ((int64_t)nchunks + nchunks0 + 2 > b.cells_cap) return cudaErrorInvalidValue;
  uint32_t* sums = b.cell_voff;
  uint32_t* offs0 = b.cell_voff + nchunks + 1;
  cudaMemsetAsync(b.cursor, 0, sizeof(uint32_t) * (size_t)(nv + 1), st);
  GM_LAUNCH(kc, "k_adj_count", st, k_adj_count<<<gs_blocks(3 * nt, 256, sms), 256, 0, st>>>(b.T, nt, b.cursor));
  GM_LAUNCH(kc, "k_row0_count", st, k_row0_count<<<nchunks0, 256, 0, st>>>(b.T, 3 * nt, offs0));
  GM_LAUNCH(kc, "k_scan_small", st, k_scan_small<<<1, 1024, 0, st>>>(offs0, nchunks0));
  GM_LAUNCH(kc, "k_row0_total", st, k_row0_total<<<1, 32, 0, st>>>(offs0, nchunks0, b.cursor));
  GM_LAUNCH(kc, "k_scan_sums", st, k_scan_sums<<<nchunks, 256, 0, st>>>(b.cursor, nv, sums));
  GM_LAUNCH(kc, "k_scan_small", st, k_scan_small<<<1, 1024, 0, st>>>(sums, nchunks));
  GM_LAUNCH(kc, "k_scan_apply", st, k_scan_apply<<<nchunks, 256, 0, st>>>(b.cursor, nv, sums, b.rowptr));
  cudaMemsetAsync(b.cursor, 0, sizeof(uint32_t) * (size_t)(nv + 1), st);
  GM_LAUNCH(kc, "k_adj_fill", st, k_adj_fill<<<gs_blocks(3 * nt, 256, sms), 256, 0, st>>>(b.T, nt, b.rowptr, b.cursor, b.adj));
  GM_LAUNCH(kc, "k_row0_fill", st, k_row0_fill<<<nchunks0, 256, 0, st>>>(b.T, 3 * nt, offs0, b.rowptr, b.adj));
  const int iters = a.bilateral_iters;
  const int zi = a.zero_isolated;
  GM_LAUNCH(kc, "k_adj_finish", st,
            k_adj_finish<<<gs_blocks(nv, 256, sms), 256, 0, st>>>(b.V, b.T, b.rowptr, b.adj, nv, zi, b.N4a,
                                                                  iters == 0 ? b.N : nullptr,
                                                                  iters > 0 ? b.ent : nullptr, b.cursor));
  if (iters > 0) {
    // the records packed: counts (in cursor) scanned into roff
    GM_LAUNCH(kc, "k_scan_sums", st, k_scan_sums<<<nchunks, 256, 0, st>>>(b.cursor, nv, sums));
    GM_LAUNCH(kc, "k_scan_small", st, k_scan_small<<<1, 1024, 0, st>>>(sums, nchunks));
    GM_LAUNCH(kc, "k_scan_apply", st, k_scan_apply<<<nchunks, 256, 0, st>>>(b.cursor, nv, sums, b.roff));
    GM_LAUNCH(kc, "k_rec_pack", st,
              k_rec_pack<<<gs_blocks(nv, 256, sms), 256, 0, st>>>(b.ent, b.rowptr, b.roff, nv, b.rec));
  }
  if (a.defer_filter) return cudaGetLastError();
  float4* nin = b.N4a;
  float4* nout = b.N4b;
  const int bil_blocks = wave_blocks(reinterpret_cast<const void*>(k_bilateral), nv, sms);
  for (int it = 0; it < iters; it++) {
    const float sn = it < 2 ? 1e10f : 0.2f;  // GMorpho.cu:6959-6969
    GM_LAUNCH(kc, "k_bilateral", st,
              k_bilateral<<<bil_blocks, 256, 0, st>>>(nin, b.roff, b.rec, nv, sn * sn, zi, nout,
                                                                   it == iters - 1 ? b.N : nullptr));
    float4* t = nin; nin = nout; nout = t;
  }
  return cudaGetLastError();
}

size_t mesh_filter_table_bytes(int n) {
  return ((sizeof(BilMesh) * (size_t)n + 15) / 16) * 16 + sizeof(int64_t) * ((size_t)n + 1);
}

cudaError_t mesh_filter_group(MeshBuffers* const* meshes, const int64_t* nv, const int* zero_isolated, int n,
                              int iters, void* table, void* h_table, int sms, cudaStream_t st, KernelCounter* kc) {
  if (iters <= 0 || n <= 0) return cudaSuccess;
  BilMesh* hm = static_cast<BilMesh*>(h_table);
  int64_t* hs = reinterpret_cast<int64_t*>(static_cast<uint8_t*>(h_table) + ((sizeof(BilMesh) * (size_t)n + 15) / 16) * 16);
  hs[0] = 0;
  for (int i = 0; i < n; i++) {
    const MeshBuffers& b = *meshes[i];
    hm[i] = BilMesh{b.N4a, b.N4b, b.roff, b.rec, b.N, zero_isolated[i]};
    hs[i + 1] = hs[i] + nv[i];
  }
  const int64_t total = hs[n];
  cudaError_t e = cudaMemcpyAsync(table, h_table, mesh_filter_table_bytes(n), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess || total == 0) return e;
  const BilMesh* dm = static_cast<const BilMesh*>(table);
  const int64_t* ds = reinterpret_cast<const int64_t*>(static_cast<const uint8_t*>(table) +
                                                       ((sizeof(BilMesh) * (size_t)n + 15) / 16) * 16);
  const int grp_blocks = wave_blocks(reinterpret_cast<const void*>(k_bilateral_group), total, sms);
  for (int it = 0; it < iters; it++) {
    const float sn = it < 2 ? 1e10f : 0.2f;  // GMorpho.cu:6959-6969
    GM_LAUNCH(kc, "k_bilateral", st,
              k_bilateral_group<<<grp_blocks, 256, 0, st>>>(dm, ds, n, it & 1, it == iters - 1, sn * sn));
  }
  return cudaGetLastError();
}

}  // namespace gm
