// serve.cu — a resident-grid edit server: brush edits of the scale field
// (ScaleField::UpdateGrid, GMorpho/ScaleField.cu:148-202) followed by a
// LOCAL re-closing and a re-mesh of the dirty region only, with continuous
// batching over several slots.  No reference counterpart: the reference
// re-closes and re-meshes the whole grid after every brush event
// (BroxyViewer.cpp:667-672).
//
// Exactness of the local re-closing.  The closing at a fine voxel depends on
// the input grid and the radii within a bounded reach (dilation r+1, erosion
// r-1, a few cells of block, contour and refinement rules), so an edit can
// change it only in a box around its brush, and a crop holding that box
// with a margin is exact on it.  plan_edit derives both margins from a host
// map of the largest radius per 8-cell brick, so that they follow the radii
// around each edit rather than the server's global bound.  Crops touching
// the grid border are aligned to it, so the border rules of the reference
// ([1, res-2] cells, data_res) act the same.
//
// Continuous batching: each slot owns a stream and a mesh buffer.  Queued
// edits are dispatched in arrival order as slots and memory free up; an edit
// whose crop overlaps the crop of an edit still on the GPU is queued behind
// it on the GPU (its stream waits for the earlier edit's write back),
// disjoint edits run concurrently.
//
// Admission by memory: an edit's crop buffers (input crop, closed crop,
// closing workspace) are sized for its own crop and taken from a device
// memory pool in stream order when it is dispatched, and returned when its
// result is collected.  An edit is dispatched only while the bytes of the
// edits on the GPU plus its own stay within the server's budget (the
// device's free memory at creation less a reserve, or the caller's); an
// edit that finds too little memory, or whose allocation fails, stays
// queued and is retried as edits finish, unless its wait passes the
// request timeout (GM_ERR_OUT_OF_MEMORY after an allocation failure,
// GM_ERR_NOT_READY otherwise).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <vector>

#include "../../include/gmorpho_gb300.h"
#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

// Largest radius of each 8-cell brick (16^3 fine voxels) of the radius
// field: one block per brick, one 16-byte row segment per thread.
constexpr int kRBrick = 8;  // cells per radius-map brick edge
__global__ void __launch_bounds__(256) k_brick_rmax(const int8_t* __restrict__ R, int n, int nb,
                                                     uint8_t* __restrict__ out) {
  const int b = blockIdx.x;
  const int bx = b % nb, by = (b / nb) % nb, bz = b / (nb * nb);
  const int fy = 2 * kRBrick * by + (threadIdx.x & 15), fz = 2 * kRBrick * bz + (threadIdx.x >> 4);
  int m = 0;
  if (fy < n && fz < n && 2 * kRBrick * bx < n) {
    const uint4 v = *reinterpret_cast<const uint4*>(R + fine_index(2 * kRBrick * bx, fy, fz, n));
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int j = 0; j < 4; j++) m = max(m, (int)(int8_t)((w[k] >> (8 * j)) & 0xffu));
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ int wm[8];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int k = 0; k < 8; k++) t = max(t, wm[k]);
    out[b] = (uint8_t)t;
  }
}

struct Box3 {
  int lo[3], hi[3];  // cells, [lo, hi)
  bool overlaps(const Box3& o) const {
    for (int a = 0; a < 3; a++)
      if (hi[a] <= o.lo[a] || o.hi[a] <= lo[a]) return false;
    return true;
  }
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr, counted = nullptr;
  cudaEvent_t written = nullptr;  // the edit's closing is in the resident grid (later overlapping edits wait on it)
  uint32_t* h_tot = nullptr;  // pinned: the crop mesh's four totals
  int phase = 0;              // 0 idle, 1 closing + counting, 2 emitting
  MeshArgs ma;
  uint8_t *Xc = nullptr, *Cc = nullptr, *ws = nullptr;  // carved from `block`
  void* block = nullptr;                                  // the edit's crop buffers (memory pool)
  int64_t bytes = 0;                                      // their size
  MeshBuffers mesh;
  bool busy = false;
  bool held = false;  // result returned by the last poll: its patch stays valid until the next poll
  uint64_t ticket = 0;
  Box3 crop, dirty;
  int cres = 0;
  double t_submit = 0.0;
  int64_t nv = 0, nt = 0;
  int status = 0;
};

struct Pending {
  uint64_t ticket;
  gm_edit edit;
  double t_submit;
  int last_fail = 0;  // GM_ERR_OUT_OF_MEMORY once an allocation for it failed
};

struct Server {
  int device = 0;
  int sms = 152;
  gm_grid_desc desc;
  const uint8_t* X = nullptr;
  int8_t* R = nullptr;
  uint8_t* C = nullptr;        // resident closing (owned)
  // resident squared lattice distance field of the input grid (owned, u16
  // per fine voxel, saturated for rmax): the input grid never changes, so
  // the dilation of any crop is a per-voxel threshold of it by the radii
  uint16_t* E = nullptr;
  uint8_t* ws_full = nullptr;  // workspace of the initial full closing
  int mode = 0;
  int rmax = 2;
  int max_cres = 0;
  // host map of an upper bound of the radius in each 8-cell brick: exact at
  // creation, raised at each dispatched brush (MAX and ZERO brushes can
  // raise radii up to their target, MIN brushes only lower them)
  std::vector<uint8_t> rmap;
  int rnb = 0;  // bricks per axis
  int bilateral = 0;
  std::vector<Slot> slots;
  cudaMemPool_t pool = nullptr;  // per-edit crop buffers
  int64_t budget = 0;            // bytes of crop buffers on the GPU at most
  int64_t inflight = 0;          // bytes of crop buffers of the edits on the GPU
  double timeout_ms = 0.0;       // longest wait in the queue (0: none)
  int inject_fail = 0;           // allocations still to fail as out of memory (fault injection)
  std::deque<Pending> queue;
  std::vector<gm_edit_result> done;
  uint64_t next_ticket = 1;
  KernelCounter* kc = nullptr;
};

constexpr int kLookAhead = 64;  // queued edits examined per dispatch round

static double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// (re)build the host radius map from the device radius field
static cudaError_t build_radius_map(Server& s) {
  s.rnb = (s.desc.res + kRBrick - 1) / kRBrick;
  const size_t nb = (size_t)s.rnb * s.rnb * s.rnb;
  s.rmap.assign(nb, 0);
  uint8_t* d_map = nullptr;
  cudaError_t e = cudaMalloc(&d_map, nb);
  if (e == cudaSuccess) {
    GM_LAUNCH(s.kc, "k_brick_rmax", 0, k_brick_rmax<<<(unsigned)nb, 256, 0, 0>>>(s.R, 2 * s.desc.res, s.rnb, d_map));
    e = cudaMemcpy(s.rmap.data(), d_map, nb, cudaMemcpyDeviceToHost);
  }
  cudaFree(d_map);
  return e;
}

struct Plan {
  Box3 dirty, crop;
  int cres;
  int rclose;  // radius bound of the crop's closing
};

// largest mapped radius over the bricks meeting the cell box [lo, hi), or
// over those of it that do not meet the box `ex` (when given)
static int map_max(const Server& s, const int lo[3], const int hi[3], const Box3* ex) {
  int b0[3], b1[3], e0[3] = {0, 0, 0}, e1[3] = {-1, -1, -1};
  for (int a = 0; a < 3; a++) {
    const int l = lo[a] < 0 ? 0 : lo[a], h = hi[a] > s.desc.res ? s.desc.res : hi[a];
    if (l >= h) return 2;
    b0[a] = l / kRBrick;
    b1[a] = (h - 1) / kRBrick;
    if (ex) {
      e0[a] = (ex->lo[a] < 0 ? 0 : ex->lo[a]) / kRBrick;
      e1[a] = ((ex->hi[a] > s.desc.res ? s.desc.res : ex->hi[a]) - 1) / kRBrick;
    }
  }
  int m = 2;
  for (int z = b0[2]; z <= b1[2]; z++)
    for (int y = b0[1]; y <= b1[1]; y++) {
      const uint8_t* row = &s.rmap[((size_t)z * s.rnb + y) * s.rnb];
      const bool in_yz = ex && z >= e0[2] && z <= e1[2] && y >= e0[1] && y <= e1[1];
      for (int x = b0[0]; x <= b1[0]; x++) {
        if (in_yz && x >= e0[0] && x <= e1[0]) continue;
        m = row[x] > m ? row[x] : m;
      }
    }
  return m;
}

// radius an edit's brush can write (upper bound), or 0 when it only lowers
static int brush_raise(const Server& s, const gm_edit& e) {
  if (e.mode == GM_BRUSH_MIN) return 0;
  const float cs_f = 0.5f * s.desc.cell_size;
  const float t = (e.mode == GM_BRUSH_ZERO ? e.global_scale : e.scale) / cs_f;
  const float c = ceilf(t);
  return c > 127.f ? 127 : (c < 0.f ? 0 : (int)c);
}

// fine-voxel box the brush kernel may change (same bounds as the kernel)
static void brush_box(const Server& s, const gm_edit& e, int lo[3], int hi[3]) {
  const float cs_f = 0.5f * s.desc.cell_size;
  const float v = e.scale;
  const float h = (e.support - v) / sqrtf(1.f - sqrtf(0.5f));
  const float reach = v + h;
  for (int a = 0; a < 3; a++) {
    lo[a] = (int)floorf((e.center[a] - reach - s.desc.bbox_min[a]) / cs_f) - 1;
    hi[a] = (int)ceilf((e.center[a] + reach - s.desc.bbox_min[a]) / cs_f) + 1;
  }
}

// Exact local re-closing plan of an edit (fine-voxel distances; r_in bounds
// the radii, old and new, in the brush cells B grown by 2, r_out those of
// the bricks around it that do not meet B + 2):
//  * the closing can change only in dirty = B + Md, Md = (r_in + 2)/2 + 4
//    cells (one block cell, one contour cell, erosion reach, refinement),
//    and at least 9 so that bricks meeting B + 2 lie inside it;
//  * the dilation of a crop is the threshold of the whole grid's distance
//    field, exact on every cell except the last layer of each open high side
//    (the tight contour rule reads the forward 2x2x2 block); the contour is
//    then exact except within two cells of an open high side and one of an
//    open low side;
//  * a cell is eroded only by sites within (r - 1)/2 + 1 cells of it, and
//    the sites outside B + 2 have radii <= r_out, so the closing is exact on
//    the cells at least (r_out + 1)/2 + 4 (erosion reach, refinement
//    neighbours, contour) from the open sides;
//  * two more cells for the mesh of the dirty box (cube corners one cell
//    past it, cubes of one more cell tagged) and two spare:
//    Mc = (r_out + 1)/2 + 8.
// Crops are cubes whose edge is a multiple of 16 cells (or the whole grid).
static bool plan_edit(const Server& s, const gm_edit& e, Plan& p) {
  const int res = s.desc.res;
  int flo[3], fhi[3];
  brush_box(s, e, flo, fhi);
  Box3 B;
  for (int a = 0; a < 3; a++) {
    B.lo[a] = (flo[a] >= 0 ? flo[a] / 2 : -((-flo[a] + 1) / 2)) - 1;  // floor(flo/2) - 1
    B.hi[a] = (fhi[a] >= 0 ? fhi[a] / 2 : -((-fhi[a] + 1) / 2)) + 2;  // floor(fhi/2) + 2
  }
  Box3 B2 = B;
  for (int a = 0; a < 3; a++) { B2.lo[a] -= 2; B2.hi[a] += 2; }
  int r_in = map_max(s, B2.lo, B2.hi, nullptr);
  const int raise = brush_raise(s, e);
  r_in = raise > r_in ? raise : r_in;
  int Md = (r_in + 2) / 2 + 4;
  Md = Md < 9 ? 9 : Md;
  const int Mc0 = s.rmax + 10;
  int rlo[3], rhi[3];
  for (int a = 0; a < 3; a++) { rlo[a] = B.lo[a] - Md - Mc0; rhi[a] = B.hi[a] + Md + Mc0; }
  const int r_out = map_max(s, rlo, rhi, &B2);
  const int rc = r_in > r_out ? r_in : r_out;
  const int Mc = (r_out + 1) / 2 + 8;
  int span = 0;
  for (int a = 0; a < 3; a++) {
    int lo = B.lo[a] - Md, hi = B.hi[a] + Md;
    lo = lo < 0 ? 0 : lo;
    hi = hi > res ? res : hi;
    if (lo >= hi) { lo = 0; hi = 0; }
    p.dirty.lo[a] = lo;
    p.dirty.hi[a] = hi;
    const int need = hi - lo + 2 * Mc;
    span = need > span ? need : span;
  }
  int cres = (span + 15) / 16 * 16;
  if (cres >= res) cres = res;
  if (cres > s.max_cres) return false;
  for (int a = 0; a < 3; a++) {
    const int room = cres - (p.dirty.hi[a] - p.dirty.lo[a]);
    int c0 = p.dirty.lo[a] - room / 2;  // centre the dirty box in the crop
    if (c0 < 0) c0 = 0;
    if (c0 + cres > res) c0 = res - cres;
    p.crop.lo[a] = c0;
    p.crop.hi[a] = c0 + cres;
  }
  p.cres = cres;
  p.rclose = cres == res ? s.rmax : (rc > s.rmax ? s.rmax : rc);
  return true;
}

// raise the radius map over the bricks the brush can change
static void map_raise(Server& s, const gm_edit& e) {
  const int raise = brush_raise(s, e);
  if (raise == 0) return;
  int flo[3], fhi[3], b0[3], b1[3];
  brush_box(s, e, flo, fhi);
  const int n = 2 * s.desc.res;
  for (int a = 0; a < 3; a++) {
    const int l = flo[a] < 0 ? 0 : flo[a], h = fhi[a] > n - 1 ? n - 1 : fhi[a];
    if (l > h) return;
    b0[a] = l / (2 * kRBrick);
    b1[a] = h / (2 * kRBrick);
  }
  for (int z = b0[2]; z <= b1[2]; z++)
    for (int y = b0[1]; y <= b1[1]; y++)
      for (int x = b0[0]; x <= b1[0]; x++) {
        uint8_t& v = s.rmap[((size_t)z * s.rnb + y) * s.rnb + x];
        v = raise > v ? (uint8_t)raise : v;
      }
}

static cudaError_t dispatch(Server& s, Slot& sl, const Pending& p, const Plan& pl, const std::vector<cudaEvent_t>& deps) {
  const gm_edit& e = p.edit;
  const int res = s.desc.res;
  const Box3& dirty = pl.dirty;
  const Box3& crop = pl.crop;
  const int cres = pl.cres;
  cudaError_t err;
  map_raise(s, e);
  sl.busy = true;
  sl.ticket = p.ticket;
  sl.crop = crop;
  sl.dirty = dirty;
  sl.cres = cres;
  sl.t_submit = p.t_submit;
  sl.status = 0;
  // overlapping edits dispatched earlier: their brush, closing and write
  // back come first (stream order on the GPU, no host round trip)
  for (cudaEvent_t d : deps) cudaStreamWaitEvent(sl.st, d, 0);
  cudaEventRecord(sl.t0, sl.st);
  // 1. brush the resident radius field (bounded box kernel)
  const float bmin[3] = {s.desc.bbox_min[0], s.desc.bbox_min[1], s.desc.bbox_min[2]};
  if ((err = launch_scale_brush(s.R, 2 * res, bmin, 0.5f * s.desc.cell_size, e.center, e.scale, e.support,
                                e.global_scale, e.mode, sl.st, s.kc)) != cudaSuccess)
    return err;
  // 2. crop the packed grid (the radius field is read in place)
  {
    const int zero[3] = {0, 0, 0};
    const int ext[3] = {cres, cres, cres};
    if ((err = launch_box_copy(s.X, res, crop.lo, sl.Xc, cres, zero, ext, sl.st, s.kc)) != cudaSuccess) return err;
  }
  // 3. close the crop
  CloseArgs a;
  a.res = cres;
  for (int k = 0; k < 3; k++) {
    int d = s.desc.data_res[k] - crop.lo[k];
    a.data_res[k] = d < 0 ? 0 : (d > cres ? cres : d);
  }
  a.X = sl.Xc;
  const int64_t N = 2 * (int64_t)res;
  a.R = s.R + 2 * crop.lo[0] + N * 2 * crop.lo[1] + N * N * 2 * crop.lo[2];
  a.r_sy = N;
  a.r_sz = N * N;
  a.uniform_r = 0;
  a.rmax = pl.rclose;
  a.mode = s.mode;
  a.se = 0;
  a.C_out = sl.Cc;
  a.D_out = nullptr;
  a.S_out = nullptr;
  a.workspace = sl.ws;
  a.num_sms = s.sms;
  a.edt = s.E + 2 * crop.lo[0] + N * 2 * crop.lo[1] + N * N * 2 * crop.lo[2];
  a.e_sy = N;
  a.e_sz = N * N;
  // only the dirty box and the two cells the mesh reads around it are used
  if (dirty.hi[0] > dirty.lo[0] && dirty.hi[1] > dirty.lo[1] && dirty.hi[2] > dirty.lo[2])
    for (int k = 0; k < 3; k++) {
      a.roi_lo[k] = dirty.lo[k] - crop.lo[k] - 2;
      a.roi_hi[k] = dirty.hi[k] - crop.lo[k] + 2;
    }
  if ((err = launch_close(a, sl.st, s.kc)) != cudaSuccess) return err;
  // 4. write back the dirty box
  {
    const int src0[3] = {dirty.lo[0] - crop.lo[0], dirty.lo[1] - crop.lo[1], dirty.lo[2] - crop.lo[2]};
    const int ext[3] = {dirty.hi[0] - dirty.lo[0], dirty.hi[1] - dirty.lo[1], dirty.hi[2] - dirty.lo[2]};
    if ((err = launch_box_copy(sl.Cc, cres, src0, s.C, res, dirty.lo, ext, sl.st, s.kc)) != cudaSuccess) return err;
  }
  cudaEventRecord(sl.written, sl.st);
  // 5. mesh the dirty box of the crop (vertices in global coordinates)
  MeshArgs ma;
  ma.res = cres;
  ma.C = sl.Cc;
  for (int k = 0; k < 3; k++) ma.bbox_min[k] = s.desc.bbox_min[k];
  ma.cell_size = s.desc.cell_size;
  ma.isovalue = 0.95f;
  ma.bilateral_iters = s.bilateral;
  ma.num_sms = s.sms;
  ma.gres = res;
  for (int k = 0; k < 3; k++) {
    ma.off[k] = crop.lo[k];
    ma.emit_lo[k] = dirty.lo[k] - crop.lo[k];
    ma.emit_hi[k] = dirty.hi[k] - crop.lo[k];
    ma.tag_lo[k] = ma.emit_lo[k];
    ma.tag_hi[k] = ma.emit_hi[k] + 1 < cres ? ma.emit_hi[k] + 1 : cres;
  }
  ma.zero_isolated = 1;
  sl.ma = ma;
  if ((err = mesh_count_launch(ma, sl.mesh, sl.st, s.kc, sl.h_tot)) != cudaSuccess) return err;
  cudaEventRecord(sl.counted, sl.st);
  sl.phase = 1;
  return cudaGetLastError();
}

// second half of an edit, once its mesh counts are on the host
static cudaError_t finish_mesh(Server& s, Slot& sl) {
  cudaError_t err;
  if ((err = mesh_count_finish(sl.mesh, sl.h_tot, &sl.nv, &sl.nt)) != cudaSuccess) return err;
  if ((err = mesh_emit(sl.ma, sl.mesh, sl.nv, sl.nt, sl.st, s.kc)) != cudaSuccess) return err;
  sl.phase = 2;
  cudaEventRecord(sl.t1, sl.st);
  return cudaGetLastError();
}

// bytes of an edit's crop buffers: the input crop, the closed crop and the
// closing workspace, each 256-byte aligned
static int64_t edit_bytes(int cres) {
  const int64_t cells = (int64_t)cres * cres * cres;
  return 2 * ((cells + 255) / 256 * 256) + (int64_t)close_workspace_bytes(cres) + 256;
}

// the slot's crop buffers back to the pool, in its stream's order
static void release_buffers(Server& s, Slot& sl) {
  if (sl.block) cudaFreeAsync(sl.block, sl.st);
  s.inflight -= sl.bytes;
  sl.block = nullptr;
  sl.Xc = sl.Cc = sl.ws = nullptr;
  sl.bytes = 0;
}

// crop buffers for an edit of crop edge cres on the slot's stream
static cudaError_t take_buffers(Server& s, Slot& sl, int cres) {
  const int64_t bytes = edit_bytes(cres);
  if (s.inject_fail > 0) {
    s.inject_fail--;
    return cudaErrorMemoryAllocation;
  }
  void* p = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(&p, (size_t)bytes, s.pool, sl.st);
  if (e != cudaSuccess) return e;
  const int64_t cells = (int64_t)cres * cres * cres, cpad = (cells + 255) / 256 * 256;
  sl.block = p;
  sl.Xc = static_cast<uint8_t*>(p);
  sl.Cc = sl.Xc + cpad;
  sl.ws = sl.Cc + cpad;
  sl.bytes = bytes;
  s.inflight += bytes;
  return cudaSuccess;
}

static void fail_slot(Server& s, Slot& sl, int status) {
  gm_edit_result r = {};
  r.ticket = sl.ticket;
  r.status = status;
  s.done.push_back(r);
  release_buffers(s, sl);
  sl.busy = false;
  sl.phase = 0;
}

static void progress(Server& s) {
  for (Slot& sl : s.slots) sl.held = false;
  // slots whose counts arrived go on to emission (no host wait)
  for (Slot& sl : s.slots) {
    if (!sl.busy || sl.phase != 1) continue;
    const cudaError_t q = cudaEventQuery(sl.counted);
    if (q == cudaErrorNotReady) continue;
    if (q != cudaSuccess || finish_mesh(s, sl) != cudaSuccess) {
      cudaGetLastError();
      fail_slot(s, sl, GM_ERR_CUDA);
    }
  }
  // collect finished slots
  for (Slot& sl : s.slots) {
    if (!sl.busy || sl.phase != 2) continue;
    const cudaError_t q = cudaEventQuery(sl.t1);
    if (q == cudaErrorNotReady) continue;
    gm_edit_result r;
    r.ticket = sl.ticket;
    r.status = q == cudaSuccess ? GM_OK : GM_ERR_CUDA;
    float dev_ms = 0.f;
    cudaEventElapsedTime(&dev_ms, sl.t0, sl.t1);
    r.device_ms = dev_ms;
    r.latency_ms = (float)(now_ms() - sl.t_submit);
    for (int a = 0; a < 3; a++) {
      r.dirty_lo[a] = 2 * sl.dirty.lo[a];
      r.dirty_hi[a] = 2 * sl.dirty.hi[a];
    }
    r.crop_res = sl.cres;
    r.patch.vertices = sl.mesh.V;
    r.patch.normals = sl.mesh.N;
    r.patch.triangles = sl.mesh.T;
    r.patch.num_vertices = sl.nv;
    r.patch.num_triangles = sl.nt;
    s.done.push_back(r);
    release_buffers(s, sl);
    sl.busy = false;
    sl.held = true;
    sl.phase = 0;
  }
  // requests that waited in the queue past the timeout
  if (s.timeout_ms > 0.0) {
    const double t = now_ms();
    for (auto it = s.queue.begin(); it != s.queue.end();) {
      if (t - it->t_submit <= s.timeout_ms) {
        ++it;
        continue;
      }
      gm_edit_result r = {};
      r.ticket = it->ticket;
      r.status = it->last_fail ? it->last_fail : GM_ERR_NOT_READY;
      r.latency_ms = (float)(t - it->t_submit);
      s.done.push_back(r);
      it = s.queue.erase(it);
    }
  }
  // Dispatch queued edits while slots are free.  An edit whose crop meets
  // the crop of an earlier edit still queued waits (its result depends on
  // that edit); later edits independent of everything queued before them go
  // ahead of it (bounded look-ahead).  One whose crop meets edits on the GPU
  // is dispatched behind them: its stream waits for their write back (its
  // brush then follows their reads of the radius field, its crop sees their
  // brushes and its write back lands after theirs).
  std::vector<Box3> waiting;  // crops of the earlier edits that stay queued
  int looked = 0;
  for (auto it = s.queue.begin(); it != s.queue.end() && looked < kLookAhead; looked++) {
    Slot* free_slot = nullptr;
    for (Slot& sl : s.slots)
      if (!sl.busy && !sl.held) { free_slot = &sl; break; }
    if (!free_slot) break;
    Plan pl;
    if (!plan_edit(s, it->edit, pl)) {
      gm_edit_result r = {};
      r.ticket = it->ticket;
      r.status = GM_ERR_CAPACITY;
      s.done.push_back(r);
      it = s.queue.erase(it);
      continue;
    }
    bool conflict = false;
    std::vector<cudaEvent_t> deps;
    for (const Slot& sl : s.slots)
      if (sl.busy && sl.crop.overlaps(pl.crop)) deps.push_back(sl.written);
    for (const Box3& w : waiting)
      if (w.overlaps(pl.crop)) conflict = true;
    if (conflict) {
      waiting.push_back(pl.crop);
      ++it;
      continue;
    }
    // admission by memory: its crop buffers must fit the budget next to
    // those of the edits on the GPU (an edit larger than the whole budget
    // is refused at once), and the allocation must succeed
    const int64_t need = edit_bytes(pl.cres);
    if (need > s.budget) {
      gm_edit_result r = {};
      r.ticket = it->ticket;
      r.status = GM_ERR_OUT_OF_MEMORY;
      s.done.push_back(r);
      it = s.queue.erase(it);
      continue;
    }
    if (s.inflight + need > s.budget || take_buffers(s, *free_slot, pl.cres) != cudaSuccess) {
      if (s.inflight + need <= s.budget) {
        cudaGetLastError();
        it->last_fail = GM_ERR_OUT_OF_MEMORY;
      }
      waiting.push_back(pl.crop);
      ++it;
      continue;
    }
    const Pending pe = *it;
    it = s.queue.erase(it);
    if (dispatch(s, *free_slot, pe, pl, deps) != cudaSuccess) {
      cudaGetLastError();
      fail_slot(s, *free_slot, GM_ERR_CUDA);
    }
  }
}

}  // namespace gm

struct gm_server {
  gm::Server s;
  gm::KernelCounter kc;
};

namespace {
bool pow2i(int v) { return v > 0 && (v & (v - 1)) == 0; }
}

extern "C" {

gm_status gm_server_create(const gm_grid_desc* desc, const uint8_t* d_input, int8_t* d_scale,
                           const gm_server_opts* opts, gm_server** out) {
  if (!desc || !d_input || !d_scale || !opts || !out) return GM_ERR_INVALID_ARGUMENT;
  if (!pow2i(desc->res) || desc->res < 16 || desc->res > 1024) return GM_ERR_INVALID_ARGUMENT;
  const bool crop_ok = opts->max_crop_res == desc->res || (opts->max_crop_res >= 16 && opts->max_crop_res % 16 == 0);
  if (opts->slots < 1 || opts->slots > 16 || !crop_ok || opts->max_crop_res > desc->res || opts->rmax < 2 ||
      opts->rmax > 127)
    return GM_ERR_INVALID_ARGUMENT;
  gm_server* srv = new gm_server();
  gm::Server& s = srv->s;
  cudaGetDevice(&s.device);
  cudaDeviceGetAttribute(&s.sms, cudaDevAttrMultiProcessorCount, s.device);
  s.desc = *desc;
  s.X = d_input;
  s.R = d_scale;
  s.mode = opts->mode;
  s.rmax = opts->rmax;
  s.max_cres = opts->max_crop_res;
  s.bilateral = opts->bilateral_iters;
  s.kc = &srv->kc;
  const size_t cells = (size_t)desc->res * desc->res * desc->res;
  cudaError_t e = cudaMalloc(&s.C, cells);
  int* d_r = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&d_r, sizeof(int));
  if (e == cudaSuccess) e = gm::launch_rmax(d_scale, (int64_t)8 * cells, d_r, s.sms, 0, s.kc);
  if (e == cudaSuccess) {
    int h = 0;
    e = cudaMemcpy(&h, d_r, sizeof(int), cudaMemcpyDeviceToHost);
    if (h > s.rmax) s.rmax = h;  // the bound must cover the field as loaded
  }
  cudaFree(d_r);
  if (e == cudaSuccess) e = gm::build_radius_map(s);
  if (e == cudaSuccess) e = cudaMalloc(&s.ws_full, gm::close_workspace_bytes(desc->res));
  if (e == cudaSuccess) e = cudaMalloc(&s.E, (size_t)8 * cells * sizeof(uint16_t));
  if (e == cudaSuccess) e = gm::launch_edt(d_input, desc->res, s.rmax, s.ws_full, s.E, 0, s.kc);
  // initial full closing of the resident grid (its dilation from the
  // distance field, like every edit's)
  if (e == cudaSuccess) {
    gm::CloseArgs a;
    a.res = desc->res;
    for (int k = 0; k < 3; k++) a.data_res[k] = desc->data_res[k];
    a.X = d_input;
    a.R = d_scale;
    a.uniform_r = 0;
    a.rmax = s.rmax;
    a.mode = s.mode;
    a.se = 0;
    a.C_out = s.C;
    a.D_out = nullptr;
    a.S_out = nullptr;
    a.workspace = s.ws_full;
    a.num_sms = s.sms;
    a.edt = s.E;
    a.e_sy = 2 * (int64_t)desc->res;
    a.e_sz = a.e_sy * a.e_sy;
    e = gm::launch_close(a, 0, s.kc);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  }
  if (s.ws_full) {
    cudaFree(s.ws_full);
    s.ws_full = nullptr;
  }
  for (int i = 0; i < opts->slots && e == cudaSuccess; i++) {
    gm::Slot sl;
    e = cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.t0);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.t1);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.counted, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.written, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_tot, 4 * sizeof(uint32_t));
    // mesh buffers for a patch of a few surface layers across the largest
    // crop, so that the first large edits do not allocate
    const int64_t nt = 16 * (int64_t)s.max_cres * s.max_cres;
    if (e == cudaSuccess) e = gm::mesh_reserve(sl.mesh, s.max_cres, nt / 2, nt);
    s.slots.push_back(sl);
  }
  // the crop buffers' pool: it keeps what it has grown to, and is grown at
  // once to what the slots need for the largest crops (within the budget),
  // so that edits do not wait for the driver
  if (e == cudaSuccess) {
    cudaMemPoolProps pp = {};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = s.device;
    e = cudaMemPoolCreate(&s.pool, &pp);
    if (e == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      e = cudaMemPoolSetAttribute(s.pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  if (e == cudaSuccess) {
    size_t free_b = 0, total_b = 0;
    e = cudaMemGetInfo(&free_b, &total_b);
    const int64_t reserve = std::max<int64_t>((int64_t)1 << 30, (int64_t)(total_b / 20));
    s.budget = std::max<int64_t>(0, (int64_t)free_b - reserve);
    const int64_t full = (int64_t)opts->slots * gm::edit_bytes(s.max_cres);
    s.budget = std::min(s.budget, full);
    void* warm = nullptr;
    if (e == cudaSuccess && s.budget > 0 && cudaMallocFromPoolAsync(&warm, (size_t)s.budget, s.pool, 0) == cudaSuccess) {
      cudaFreeAsync(warm, 0);
      e = cudaStreamSynchronize(0);
    }
    cudaGetLastError();
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    gm_server_destroy(srv);
    return e == cudaErrorMemoryAllocation ? GM_ERR_OUT_OF_MEMORY : GM_ERR_CUDA;
  }
  *out = srv;
  return GM_OK;
}

gm_status gm_server_destroy(gm_server* srv) {
  if (!srv) return GM_ERR_INVALID_ARGUMENT;
  gm::Server& s = srv->s;
  cudaSetDevice(s.device);
  for (gm::Slot& sl : s.slots) {
    if (sl.st) cudaStreamSynchronize(sl.st);
    if (sl.st) cudaStreamDestroy(sl.st);
    if (sl.t0) cudaEventDestroy(sl.t0);
    if (sl.t1) cudaEventDestroy(sl.t1);
    if (sl.counted) cudaEventDestroy(sl.counted);
    if (sl.written) cudaEventDestroy(sl.written);
    if (sl.h_tot) cudaFreeHost(sl.h_tot);
    if (sl.block) cudaFree(sl.block);
    sl.mesh.release();
  }
  if (s.pool) {
    cudaDeviceSynchronize();
    cudaMemPoolDestroy(s.pool);
  }
  cudaFree(s.C);
  cudaFree(s.E);
  cudaFree(s.ws_full);
  srv->kc.release();
  delete srv;
  return GM_OK;
}

gm_status gm_server_submit(gm_server* srv, const gm_edit* edit, uint64_t* ticket) {
  if (!srv || !edit) return GM_ERR_INVALID_ARGUMENT;
  if (edit->mode != GM_BRUSH_MAX && edit->mode != GM_BRUSH_MIN && edit->mode != GM_BRUSH_ZERO)
    return GM_ERR_INVALID_ARGUMENT;
  const float cs_f = 0.5f * srv->s.desc.cell_size;
  const int r_new = (int)floorf(edit->scale / cs_f);
  const int r_zero = (int)floorf(edit->global_scale / cs_f);
  if (r_new > srv->s.rmax || (edit->mode == GM_BRUSH_ZERO && r_zero > srv->s.rmax))
    return GM_ERR_CAPACITY;  // a radius above the server's bound would break the local re-closing
  gm::Pending p{srv->s.next_ticket++, *edit, gm::now_ms()};
  srv->s.queue.push_back(p);
  if (ticket) *ticket = p.ticket;
  cudaSetDevice(srv->s.device);
  gm::progress(srv->s);
  return GM_OK;
}

gm_status gm_server_poll(gm_server* srv, gm_edit_result* results, int32_t cap, int32_t* count) {
  if (!srv || !count || (cap > 0 && !results)) return GM_ERR_INVALID_ARGUMENT;
  cudaSetDevice(srv->s.device);
  gm::progress(srv->s);
  int n = 0;
  while (n < cap && !srv->s.done.empty()) {
    results[n++] = srv->s.done.front();
    srv->s.done.erase(srv->s.done.begin());
  }
  *count = n;
  return GM_OK;
}

int32_t gm_server_pending(gm_server* srv) {
  if (!srv) return -1;
  int n = (int)srv->s.queue.size();
  for (const gm::Slot& sl : srv->s.slots) n += sl.busy ? 1 : 0;
  return n;
}

const uint8_t* gm_server_closing(gm_server* srv) { return srv ? srv->s.C : nullptr; }

long long gm_server_kernel_launches(gm_server* srv) { return srv ? srv->kc.launches : -1; }

gm_status gm_server_snapshot(gm_server* srv, uint8_t* h_closing, int8_t* h_scale) {
  if (!srv || (!h_closing && !h_scale)) return GM_ERR_INVALID_ARGUMENT;
  gm::Server& s = srv->s;
  if (gm_server_pending(srv) != 0) return GM_ERR_NOT_READY;
  cudaSetDevice(s.device);
  const size_t cells = (size_t)s.desc.res * s.desc.res * s.desc.res;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess && h_closing) e = cudaMemcpy(h_closing, s.C, cells, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && h_scale) e = cudaMemcpy(h_scale, s.R, 8 * cells, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? GM_OK : GM_ERR_CUDA;
}

gm_status gm_server_restore(gm_server* srv, const uint8_t* h_closing, const int8_t* h_scale) {
  if (!srv || !h_closing || !h_scale) return GM_ERR_INVALID_ARGUMENT;
  gm::Server& s = srv->s;
  if (gm_server_pending(srv) != 0) return GM_ERR_NOT_READY;
  cudaSetDevice(s.device);
  const size_t cells = (size_t)s.desc.res * s.desc.res * s.desc.res;
  cudaError_t e = cudaDeviceSynchronize();
  int* d_r = nullptr;
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(s.R, h_scale, 8 * cells, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&d_r, sizeof(int));
  if (e == cudaSuccess) e = gm::launch_rmax(s.R, (int64_t)8 * cells, d_r, s.sms, 0, s.kc);
  if (e == cudaSuccess) e = cudaMemcpy(&h, d_r, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d_r);
  if (e != cudaSuccess) return GM_ERR_CUDA;
  if (h > s.rmax) return GM_ERR_CAPACITY;  // the field is in place but edits need a larger bound
  e = cudaMemcpy(s.C, h_closing, cells, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = gm::build_radius_map(s);
  return e == cudaSuccess ? GM_OK : GM_ERR_CUDA;
}

gm_status gm_server_set_admission(gm_server* srv, int64_t budget_bytes, float timeout_ms) {
  if (!srv || timeout_ms < 0.f) return GM_ERR_INVALID_ARGUMENT;
  if (budget_bytes > 0) srv->s.budget = budget_bytes;
  srv->s.timeout_ms = timeout_ms;
  return GM_OK;
}

gm_status gm_server_memory(gm_server* srv, int64_t* inflight_bytes, int64_t* budget_bytes) {
  if (!srv) return GM_ERR_INVALID_ARGUMENT;
  if (inflight_bytes) *inflight_bytes = srv->s.inflight;
  if (budget_bytes) *budget_bytes = srv->s.budget;
  return GM_OK;
}

gm_status gm_server_inject_alloc_failures(gm_server* srv, int32_t count) {
  if (!srv || count < 0) return GM_ERR_INVALID_ARGUMENT;
  srv->s.inject_fail = count;
  return GM_OK;
}

gm_status gm_server_profile(gm_server* srv, int32_t enable) {
  if (!srv) return GM_ERR_INVALID_ARGUMENT;
  cudaSetDevice(srv->s.device);
  srv->kc.flush();
  srv->kc.totals.clear();
  srv->kc.profiling = enable != 0;
  return GM_OK;
}

int64_t gm_server_profile_read(gm_server* srv, char* buf, int64_t cap) {
  if (!srv) return -1;
  cudaSetDevice(srv->s.device);
  return gm::profile_json(srv->kc, buf, cap);
}

}  // extern "C"
