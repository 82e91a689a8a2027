// serve.cu — a resident-grid edit server: brush edits of the scale field
// (ScaleField::UpdateGrid, GMorpho/ScaleField.cu:148-202) followed by a
// LOCAL re-closing and a re-mesh of the dirty region only, with continuous
// batching over several slots.  No reference counterpart: the reference
// re-closes and re-meshes the whole grid after every brush event
// (BroxyViewer.cpp:667-672).
//
// Exactness of the local re-closing.  The closing at a fine voxel depends on
// the input grid and radii within (rmax+1) (dilation reach) + (rmax-1)
// (erosion reach) fine voxels plus a few cells of contour tagging.  An edit
// that changes radii inside box B can therefore only change the closing
// inside A = B grown by M, and the closing on A is computed exactly from a
// crop holding A grown by M again, M = 2 rmax + 8 fine voxels (cell
// aligned).  Crops touching the grid border are aligned to it, so the
// border rules of the reference ([1, res-2] cells, data_res) act the same.
//
// Continuous batching: each slot owns a stream, crop buffers and a mesh
// buffer.  Queued edits are dispatched in arrival order as slots free up; an
// edit whose crop overlaps the crop of an edit still on the GPU waits (its
// result depends on the earlier one), disjoint edits run concurrently.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <deque>
#include <vector>

#include "../../include/gmorpho_gb300.h"
#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

// crop of the packed grid (cells) and of the radius field (fine voxels);
// outside the source grid: empty cells, radius 0
__global__ void k_crop(const uint8_t* __restrict__ X, const int8_t* __restrict__ R, int res, int cx0, int cy0,
                       int cz0, int cres, uint8_t* __restrict__ Xc, int8_t* __restrict__ Rc) {
  const int64_t cells = (int64_t)cres * cres * cres;
  const int N = 2 * res, cN = 2 * cres;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cells; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % cres), y = (int)((i / cres) % cres), z = (int)(i / ((int64_t)cres * cres));
    const int gx = cx0 + x, gy = cy0 + y, gz = cz0 + z;
    const bool in = gx >= 0 && gy >= 0 && gz >= 0 && gx < res && gy < res && gz < res;
    Xc[i] = in ? X[cell_index(gx, gy, gz, res)] : (uint8_t)0;
    for (int k = 0; k < 8; k++) {
      const int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
      Rc[fine_index(fx, fy, fz, cN)] = in ? R[fine_index(2 * gx + (k & 1), 2 * gy + ((k >> 1) & 1), 2 * gz + (k >> 2), N)]
                                          : (int8_t)0;
    }
  }
}

// write the crop's closing back on the dirty box of cells [lo, hi)
__global__ void k_writeback(const uint8_t* __restrict__ Cc, int cres, int cx0, int cy0, int cz0, uint8_t* __restrict__ C,
                            int res, int lx, int ly, int lz, int hx, int hy, int hz) {
  const int wx = hx - lx, wy = hy - ly, wz = hz - lz;
  const int64_t total = (int64_t)wx * wy * wz;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = lx + (int)(i % wx), y = ly + (int)((i / wx) % wy), z = lz + (int)(i / ((int64_t)wx * wy));
    C[cell_index(x, y, z, res)] = Cc[cell_index(x - cx0, y - cy0, z - cz0, cres)];
  }
}

// 1 for the triangles of the crop mesh whose centroid lies in the dirty box
// (fine-voxel units relative to the crop origin): the patch of this edit
__global__ void k_patch_mask(const float* __restrict__ V, const uint32_t* __restrict__ T, int64_t nt, float ox,
                             float oy, float oz, float inv_cs, float lx, float ly, float lz, float hx, float hy,
                             float hz, uint8_t* __restrict__ keep) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
    float c[3] = {0.f, 0.f, 0.f};
    for (int j = 0; j < 3; j++) {
      const uint32_t v = T[3 * t + j];
      c[0] += V[3 * (size_t)v];
      c[1] += V[3 * (size_t)v + 1];
      c[2] += V[3 * (size_t)v + 2];
    }
    const float x = (c[0] / 3.f - ox) * inv_cs, y = (c[1] / 3.f - oy) * inv_cs, z = (c[2] / 3.f - oz) * inv_cs;
    keep[t] = (x >= lx && x < hx && y >= ly && y < hy && z >= lz && z < hz) ? 1 : 0;
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
  uint32_t* h_tot = nullptr;  // pinned: the crop mesh's four totals
  int phase = 0;              // 0 idle, 1 closing + counting, 2 emitting
  MeshArgs ma;
  uint8_t *Xc = nullptr, *Cc = nullptr, *ws = nullptr, *keep = nullptr;
  int8_t* Rc = nullptr;
  size_t keep_cap = 0;
  MeshBuffers mesh;
  bool busy = false;
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
};

struct Server {
  int device = 0;
  int sms = 152;
  gm_grid_desc desc;
  const uint8_t* X = nullptr;
  int8_t* R = nullptr;
  uint8_t* C = nullptr;        // resident closing (owned)
  uint8_t* ws_full = nullptr;  // workspace of the initial full closing
  int mode = 0;
  int rmax = 2;
  int max_cres = 0;
  int bilateral = 0;
  std::vector<Slot> slots;
  std::deque<Pending> queue;
  std::vector<gm_edit_result> done;
  uint64_t next_ticket = 1;
  KernelCounter* kc = nullptr;
};

static double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static int margin_cells(int rmax) { return (2 * rmax + 8 + 1) / 2 + 1; }

// dirty box and crop of an edit; false when it needs a crop above max_cres
static bool plan_edit(const Server& s, const gm_edit& e, Box3& dirty, Box3& crop, int& cres) {
  const int res = s.desc.res;
  const float cs_f = 0.5f * s.desc.cell_size;  // fine voxel size (scale-field cell)
  const float v = e.scale;
  const float h = (e.support - v) / sqrtf(1.f - sqrtf(0.5f));
  const float reach = v + h;
  const int M = margin_cells(s.rmax);
  int span = 0;
  for (int a = 0; a < 3; a++) {
    const float lo = (e.center[a] - reach - s.desc.bbox_min[a]) / cs_f;
    const float hi = (e.center[a] + reach - s.desc.bbox_min[a]) / cs_f;
    int blo = (int)floorf(lo) / 2 - 1, bhi = (int)ceilf(hi) / 2 + 2;  // brush box in cells
    dirty.lo[a] = blo - M < 0 ? 0 : blo - M;
    dirty.hi[a] = bhi + M > res ? res : bhi + M;
    if (dirty.lo[a] >= dirty.hi[a]) { dirty.lo[a] = 0; dirty.hi[a] = 0; }
    const int need = dirty.hi[a] - dirty.lo[a] + 2 * M;
    span = need > span ? need : span;
  }
  cres = 16;
  while (cres < span) cres *= 2;
  if (cres > res) cres = res;
  if (cres > s.max_cres) return false;
  for (int a = 0; a < 3; a++) {
    int c0 = dirty.lo[a] - M;
    const int room = cres - (dirty.hi[a] - dirty.lo[a]);
    c0 = dirty.lo[a] - room / 2;  // centre the dirty box in the crop
    if (c0 < 0) c0 = 0;
    if (c0 + cres > res) c0 = res - cres;
    crop.lo[a] = c0;
    crop.hi[a] = c0 + cres;
  }
  return true;
}

static cudaError_t dispatch(Server& s, Slot& sl, const Pending& p, const Box3& dirty, const Box3& crop, int cres) {
  const gm_edit& e = p.edit;
  cudaError_t err;
  sl.busy = true;
  sl.ticket = p.ticket;
  sl.crop = crop;
  sl.dirty = dirty;
  sl.cres = cres;
  sl.t_submit = p.t_submit;
  sl.status = 0;
  cudaEventRecord(sl.t0, sl.st);
  // 1. brush the resident radius field (bounded box kernel)
  const float bmin[3] = {s.desc.bbox_min[0], s.desc.bbox_min[1], s.desc.bbox_min[2]};
  if ((err = launch_scale_brush(s.R, 2 * s.desc.res, bmin, 0.5f * s.desc.cell_size, e.center, e.scale, e.support,
                                e.global_scale, e.mode, sl.st, s.kc)) != cudaSuccess)
    return err;
  // 2. crop, 3. close the crop
  const int64_t ccells = (int64_t)cres * cres * cres;
  int blocks = (int)((ccells + 255) / 256);
  if (blocks > s.sms * 32) blocks = s.sms * 32;
  GM_LAUNCH(s.kc, "k_crop", sl.st,
            k_crop<<<blocks, 256, 0, sl.st>>>(s.X, s.R, s.desc.res, crop.lo[0], crop.lo[1], crop.lo[2], cres, sl.Xc,
                                              sl.Rc));
  CloseArgs a;
  a.res = cres;
  for (int k = 0; k < 3; k++) {
    int d = s.desc.data_res[k] - crop.lo[k];
    a.data_res[k] = d < 0 ? 0 : (d > cres ? cres : d);
  }
  a.X = sl.Xc;
  a.R = sl.Rc;
  a.uniform_r = 0;
  a.rmax = s.rmax;
  a.mode = s.mode;
  a.se = 0;
  a.C_out = sl.Cc;
  a.D_out = nullptr;
  a.S_out = nullptr;
  a.workspace = sl.ws;
  a.num_sms = s.sms;
  if ((err = launch_close(a, sl.st, s.kc)) != cudaSuccess) return err;
  // 4. write back the dirty box
  const int64_t dcells = (int64_t)(dirty.hi[0] - dirty.lo[0]) * (dirty.hi[1] - dirty.lo[1]) * (dirty.hi[2] - dirty.lo[2]);
  if (dcells > 0) {
    int b2 = (int)((dcells + 255) / 256);
    if (b2 > s.sms * 32) b2 = s.sms * 32;
    GM_LAUNCH(s.kc, "k_writeback", sl.st,
              k_writeback<<<b2, 256, 0, sl.st>>>(sl.Cc, cres, crop.lo[0], crop.lo[1], crop.lo[2], s.C, s.desc.res,
                                                 dirty.lo[0], dirty.lo[1], dirty.lo[2], dirty.hi[0], dirty.hi[1],
                                                 dirty.hi[2]));
  }
  // 5. re-mesh the crop; the dirty box's triangles form the patch
  MeshArgs ma;
  ma.res = cres;
  ma.C = sl.Cc;
  for (int k = 0; k < 3; k++) ma.bbox_min[k] = s.desc.bbox_min[k] + crop.lo[k] * s.desc.cell_size;
  ma.cell_size = s.desc.cell_size;
  ma.isovalue = 0.95f;
  ma.bilateral_iters = s.bilateral;
  ma.num_sms = s.sms;
  sl.ma = ma;
  if ((err = mesh_count_launch(ma, sl.mesh, sl.st, s.kc, sl.h_tot)) != cudaSuccess) return err;
  cudaEventRecord(sl.counted, sl.st);
  sl.phase = 1;
  return cudaGetLastError();
}

// second half of an edit, once its mesh counts are on the host
static cudaError_t finish_mesh(Server& s, Slot& sl) {
  cudaError_t err;
  const Box3& dirty = sl.dirty;
  const Box3& crop = sl.crop;
  if ((err = mesh_count_finish(sl.mesh, sl.h_tot, &sl.nv, &sl.nt)) != cudaSuccess) return err;
  if ((err = mesh_emit(sl.ma, sl.mesh, sl.nv, sl.nt, sl.st, s.kc)) != cudaSuccess) return err;
  if ((size_t)sl.nt > sl.keep_cap) {
    cudaFree(sl.keep);
    sl.keep = nullptr;
    sl.keep_cap = 0;
    if ((err = cudaMalloc(&sl.keep, (size_t)sl.nt + 1024)) != cudaSuccess) return err;
    sl.keep_cap = (size_t)sl.nt + 1024;
  }
  if (sl.nt > 0) {
    const float cs_f = 0.5f * s.desc.cell_size;
    int b3 = (int)((sl.nt + 255) / 256);
    if (b3 > s.sms * 32) b3 = s.sms * 32;
    GM_LAUNCH(s.kc, "k_patch_mask", sl.st,
              k_patch_mask<<<b3, 256, 0, sl.st>>>(sl.mesh.V, sl.mesh.T, sl.nt, sl.ma.bbox_min[0], sl.ma.bbox_min[1],
                                                  sl.ma.bbox_min[2], 1.f / cs_f, 2.f * (dirty.lo[0] - crop.lo[0]),
                                                  2.f * (dirty.lo[1] - crop.lo[1]), 2.f * (dirty.lo[2] - crop.lo[2]),
                                                  2.f * (dirty.hi[0] - crop.lo[0]), 2.f * (dirty.hi[1] - crop.lo[1]),
                                                  2.f * (dirty.hi[2] - crop.lo[2]), sl.keep));
  }
  sl.phase = 2;
  cudaEventRecord(sl.t1, sl.st);
  return cudaGetLastError();
}

static void fail_slot(Server& s, Slot& sl, int status) {
  gm_edit_result r = {};
  r.ticket = sl.ticket;
  r.status = status;
  s.done.push_back(r);
  sl.busy = false;
  sl.phase = 0;
}

static void progress(Server& s) {
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
    r.patch.vertices = sl.mesh.V;
    r.patch.normals = sl.mesh.N;
    r.patch.triangles = sl.mesh.T;
    r.patch.num_vertices = sl.nv;
    r.patch.num_triangles = sl.nt;
    r.patch_keep = sl.keep;
    s.done.push_back(r);
    sl.busy = false;
    sl.phase = 0;
  }
  // dispatch queued edits in order while slots are free and crops disjoint
  while (!s.queue.empty()) {
    const Pending& p = s.queue.front();
    Box3 dirty, crop;
    int cres;
    if (!plan_edit(s, p.edit, dirty, crop, cres)) {
      gm_edit_result r = {};
      r.ticket = p.ticket;
      r.status = GM_ERR_CAPACITY;
      s.done.push_back(r);
      s.queue.pop_front();
      continue;
    }
    bool conflict = false;
    Slot* free_slot = nullptr;
    for (Slot& sl : s.slots) {
      if (sl.busy && sl.crop.overlaps(crop)) conflict = true;
      if (!sl.busy && !free_slot) free_slot = &sl;
    }
    if (conflict || !free_slot) break;
    const Pending pe = p;
    s.queue.pop_front();
    if (dispatch(s, *free_slot, pe, dirty, crop, cres) != cudaSuccess) {
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
  if (opts->slots < 1 || opts->slots > 16 || !pow2i(opts->max_crop_res) || opts->max_crop_res < 16 ||
      opts->max_crop_res > desc->res || opts->rmax < 2 || opts->rmax > 127)
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
  if (e == cudaSuccess) e = cudaMalloc(&s.ws_full, gm::close_workspace_bytes(desc->res));
  // initial full closing of the resident grid
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
    e = gm::launch_close(a, 0, s.kc);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  }
  if (s.ws_full) {
    cudaFree(s.ws_full);
    s.ws_full = nullptr;
  }
  const size_t ccells = (size_t)s.max_cres * s.max_cres * s.max_cres;
  for (int i = 0; i < opts->slots && e == cudaSuccess; i++) {
    gm::Slot sl;
    e = cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.t0);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.t1);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.counted, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_tot, 4 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&sl.Xc, ccells);
    if (e == cudaSuccess) e = cudaMalloc(&sl.Cc, ccells);
    if (e == cudaSuccess) e = cudaMalloc(&sl.Rc, 8 * ccells);
    if (e == cudaSuccess) e = cudaMalloc(&sl.ws, gm::close_workspace_bytes(s.max_cres));
    s.slots.push_back(sl);
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
    if (sl.h_tot) cudaFreeHost(sl.h_tot);
    cudaFree(sl.Xc);
    cudaFree(sl.Cc);
    cudaFree(sl.Rc);
    cudaFree(sl.ws);
    cudaFree(sl.keep);
    sl.mesh.release();
  }
  cudaFree(s.C);
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

}  // extern "C"
