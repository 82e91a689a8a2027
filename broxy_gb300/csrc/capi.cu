// capi.cu — the extern "C" boundary of libgmorpho_gb300 (gmorpho_gb300.h).
//
// Validates arguments, owns cached device workspaces per context, turns
// CUDA errors into gm_status codes (never aborts), and counts the kernels it
// launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gmorpho_gb300.h"
#include "gm_common.cuh"
#include "tma.cuh"
#include "gm_internal.h"

namespace gm {

cudaError_t ensure_dynamic_smem(const void* kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> set;  // (kernel, device) -> limit set
  std::lock_guard<std::mutex> lock(mu);
  size_t& have = set[{kernel, dev}];
  if (have >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) have = bytes;
  return e;
}

cudaEvent_t KernelCounter::start(cudaStream_t st) {
  cudaEvent_t e;
  if (!pool.empty()) {
    e = pool.back();
    pool.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    return nullptr;
  }
  cudaEventRecord(e, st);
  return e;
}

void KernelCounter::stop(const char* name, cudaStream_t st, cudaEvent_t a) {
  launches++;
  if (!profiling || a == nullptr) return;
  cudaEvent_t b;
  if (!pool.empty()) {
    b = pool.back();
    pool.pop_back();
  } else if (cudaEventCreate(&b) != cudaSuccess) {
    pool.push_back(a);
    return;
  }
  cudaEventRecord(b, st);
  pending.push_back(Pending{name, a, b});
  if (pending.size() > 4096) flush();
}

void KernelCounter::flush() {
  for (const Pending& p : pending) {
    cudaEventSynchronize(p.b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    auto& t = totals[p.name];
    t.first += 1;
    t.second += ms;
    pool.push_back(p.a);
    pool.push_back(p.b);
  }
  pending.clear();
}

int64_t profile_json(KernelCounter& kc, char* buf, int64_t cap) {
  kc.flush();
  std::string js = "{";
  bool first = true;
  for (const auto& kv : kc.totals) {
    char tmp[256];
    snprintf(tmp, sizeof(tmp), "%s\"%s\": {\"launches\": %lld, \"ms\": %.6f}", first ? "" : ", ", kv.first.c_str(),
             kv.second.first, kv.second.second);
    js += tmp;
    first = false;
  }
  js += "}";
  const int64_t need = (int64_t)js.size() + 1;
  if (buf && cap >= need) memcpy(buf, js.c_str(), (size_t)need);
  return need;
}

void KernelCounter::release() {
  flush();
  for (cudaEvent_t e : pool) cudaEventDestroy(e);
  pool.clear();
}

}  // namespace gm

struct gm_ctx {
  int device = 0;
  int num_sms = 152;
  std::string last_error;
  gm::KernelCounter kc;
  // closing workspace
  uint8_t* ws = nullptr;
  size_t ws_bytes = 0;
  // gm_update staging
  uint8_t* d_X = nullptr;
  size_t X_bytes = 0;
  int8_t* d_R = nullptr;
  size_t R_bytes = 0;
  uint8_t* d_C = nullptr;
  size_t C_bytes = 0;
  int* d_int = nullptr;
  // voxelizer scratch
  uint8_t* vox = nullptr;
  uint8_t* rmap = nullptr;  // 16^3-block radius map of the last radius field
  size_t rmap_bytes = 0;
  size_t vox_bytes = 0;
  // batched closing + meshing state (lanes, per-instance meshes, graph)
  void* batch = nullptr;
  // host-buffer updates: a copy stream and its events
  cudaStream_t copy_st = nullptr;
  cudaEvent_t ev_copy = nullptr, ev_geom = nullptr;
  // the radius field's upload in z slabs: one event per slab copied and per
  // slab bound read back, the bounds in pinned memory
  static constexpr int kSlabs = 8;
  cudaEvent_t ev_slab[kSlabs] = {}, ev_max[kSlabs] = {};
  int* h_slab = nullptr;
  // last mesh
  gm::MeshBuffers mesh;
  int64_t nv = 0, nt = 0;
  bool has_mesh = false;
};

namespace {

gm_status fail(gm_ctx* ctx, gm_status s, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return s;
}

gm_status cuda_fail(gm_ctx* ctx, cudaError_t e, const char* where) {
  const gm_status s = e == cudaErrorMemoryAllocation ? GM_ERR_OUT_OF_MEMORY : GM_ERR_CUDA;
  return fail(ctx, s, std::string(where) + ": " + cudaGetErrorString(e));
}

#define GM_CHECK_CUDA(ctx, expr, where)              \
  do {                                               \
    cudaError_t e_ = (expr);                         \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, where); \
  } while (0)

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

gm_status check_desc(gm_ctx* ctx, const gm_grid_desc* d) {
  if (!d) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "grid descriptor is NULL");
  if (!pow2(d->res) || d->res < 16 || d->res > 1024)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "res must be a power of two in [16, 1024], got " + std::to_string(d->res));
  for (int a = 0; a < 3; a++)
    if (d->data_res[a] < 0 || d->data_res[a] > d->res)
      return fail(ctx, GM_ERR_INVALID_ARGUMENT, "data_res must lie in [0, res]");
  return GM_OK;
}

gm_status ensure(gm_ctx* ctx, void** p, size_t& have, size_t need, const char* what) {
  if (have >= need && *p) return GM_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  have = 0;
  cudaError_t e = cudaMalloc(p, need);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, e == cudaErrorMemoryAllocation ? GM_ERR_OUT_OF_MEMORY : GM_ERR_CUDA,
                std::string("allocating ") + what + " (" + std::to_string(need) + " bytes): " + cudaGetErrorString(e));
  }
  have = need;
  return GM_OK;
}

gm_status set_device(gm_ctx* ctx) {
  GM_CHECK_CUDA(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  return GM_OK;
}

}  // namespace

extern "C" {

const char* gm_status_string(gm_status s) {
  switch (s) {
    case GM_OK: return "ok";
    case GM_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GM_ERR_CUDA: return "CUDA error";
    case GM_ERR_OUT_OF_MEMORY: return "out of device memory";
    case GM_ERR_UNSUPPORTED: return "unsupported";
    case GM_ERR_CAPACITY: return "capacity exceeded";
    case GM_ERR_NOT_READY: return "not ready";
  }
  return "unknown status";
}

int gm_abi_version(void) { return GM_ABI_VERSION; }

gm_status gm_ctx_create(int device, gm_ctx** out) {
  if (!out) return GM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) { cudaGetLastError(); return GM_ERR_CUDA; }
  if (device < 0 || device >= n) return GM_ERR_INVALID_ARGUMENT;
  gm_ctx* c = new gm_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess) { delete c; return GM_ERR_CUDA; }
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaMalloc(&c->d_int, 16 * sizeof(int)) != cudaSuccess) { delete c; return GM_ERR_OUT_OF_MEMORY; }
  gm::tma_init();
  *out = c;
  return GM_OK;
}

gm_status gm_ctx_destroy(gm_ctx* ctx) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaFree(ctx->ws);
  cudaFree(ctx->d_X);
  cudaFree(ctx->d_R);
  cudaFree(ctx->d_C);
  cudaFree(ctx->d_int);
  cudaFree(ctx->rmap);
  cudaFree(ctx->vox);
  if (ctx->copy_st) cudaStreamDestroy(ctx->copy_st);
  if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
  if (ctx->ev_geom) cudaEventDestroy(ctx->ev_geom);
  for (int k = 0; k < gm_ctx::kSlabs; k++) {
    if (ctx->ev_slab[k]) cudaEventDestroy(ctx->ev_slab[k]);
    if (ctx->ev_max[k]) cudaEventDestroy(ctx->ev_max[k]);
  }
  if (ctx->h_slab) cudaFreeHost(ctx->h_slab);
  ctx->mesh.release();
  gm::batch_release(ctx->batch);
  ctx->kc.release();
  delete ctx;
  return GM_OK;
}

const char* gm_ctx_last_error(const gm_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "NULL context"; }

long long gm_ctx_kernel_launches(const gm_ctx* ctx) { return ctx ? ctx->kc.launches : -1; }

gm_status gm_kernel_error_flags(uint32_t* flags, int32_t clear) {
  if (!flags) return GM_ERR_INVALID_ARGUMENT;
  unsigned int f = 0;
  if (cudaDeviceSynchronize() != cudaSuccess || gm::kernel_error_flags(&f, clear != 0) != cudaSuccess) {
    cudaGetLastError();
    return GM_ERR_CUDA;
  }
  *flags = f;
  return GM_OK;
}

gm_status gm_ctx_profile(gm_ctx* ctx, int32_t enable) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  ctx->kc.flush();
  ctx->kc.profiling = enable != 0;
  return GM_OK;
}

gm_status gm_ctx_profile_reset(gm_ctx* ctx) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  ctx->kc.flush();
  ctx->kc.totals.clear();
  return GM_OK;
}

int64_t gm_ctx_profile_read(gm_ctx* ctx, char* buf, int64_t cap) {
  if (!ctx) return -1;
  return gm::profile_json(ctx->kc, buf, cap);
}

// ------------------------------------------------------------------ a2

gm_status gm_grid_attributes(const float* P, int64_t nv, int32_t base_res, float margin, gm_grid_desc* out) {
  if (!P || nv <= 0 || !out || !pow2(base_res) || base_res < 16 || base_res > 1024) return GM_ERR_INVALID_ARGUMENT;
  float mn[3] = {P[0], P[1], P[2]}, mx[3] = {P[0], P[1], P[2]};
  for (int64_t i = 0; i < nv; i++)
    for (int a = 0; a < 3; a++) {
      const float v = P[3 * i + a];
      if (v < mn[a]) mn[a] = v;
      if (v > mx[a]) mx[a] = v;
    }
  const float ext = std::fmax(std::fabs(mx[0] - mn[0]), std::fmax(std::fabs(mx[1] - mn[1]), std::fabs(mx[2] - mn[2])));
  const float thickness = ext / (float)base_res;
  const float off = 2.f * thickness + margin;
  for (int a = 0; a < 3; a++) { mn[a] -= off; mx[a] += off; }
  const float c = std::fmax(std::fabs(mx[0] - mn[0]), std::fmax(std::fabs(mx[1] - mn[1]), std::fabs(mx[2] - mn[2]))) /
                  (float)base_res;
  for (int a = 0; a < 3; a++) {
    out->bbox_min[a] = mn[a];
    out->bbox_max[a] = mx[a];
    out->data_res[a] = (int32_t)std::ceil((mx[a] - mn[a]) / c);
    if (out->data_res[a] > base_res) out->data_res[a] = base_res;
  }
  out->res = base_res;
  out->cell_size = c;
  return GM_OK;
}

gm_status gm_voxelize(gm_ctx* ctx, const gm_grid_desc* desc, const float* d_points, int64_t num_points,
                      const uint32_t* d_triangles, int64_t num_triangles, uint8_t* d_grid, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!d_grid || (num_triangles > 0 && (!d_points || !d_triangles)) || num_points < 0 || num_triangles < 0)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_voxelize: NULL buffer or negative count");
  if ((s = set_device(ctx)) != GM_OK) return s;
  if ((s = ensure(ctx, (void**)&ctx->vox, ctx->vox_bytes, gm::voxelize_scratch_bytes(desc->res), "voxelizer scratch")) !=
      GM_OK)
    return s;
  GM_CHECK_CUDA(ctx,
                gm::launch_voxelize(d_points, num_points, d_triangles, num_triangles, desc->res, desc->bbox_min,
                                    desc->cell_size, d_grid, ctx->vox, (cudaStream_t)stream, &ctx->kc),
                "gm_voxelize");
  return GM_OK;
}

// ------------------------------------------------------------------ a3

__global__ void k_fill_i8(int8_t* p, int64_t n, int8_t v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

gm_status gm_scalefield_fill(gm_ctx* ctx, int8_t* d_scale, int64_t n, int32_t value, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  if (!d_scale || n < 0) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_scalefield_fill: bad buffer");
  gm_status s = set_device(ctx);
  if (s != GM_OK) return s;
  // cudaMemset stores the low byte of the value (GMorpho/ScaleField.cu:143-146)
  GM_CHECK_CUDA(ctx, cudaMemsetAsync(d_scale, value & 0xff, (size_t)n, (cudaStream_t)stream), "gm_scalefield_fill");
  return GM_OK;
}

gm_status gm_scalefield_brush(gm_ctx* ctx, int8_t* d_scale, int32_t fine_res, const float* bbox_min, float cell_size,
                              const float* position, float scale, float support, float global_scale,
                              gm_brush_mode mode, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  if (!d_scale || !bbox_min || !position || fine_res <= 0 || !(cell_size > 0))
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_scalefield_brush: bad argument");
  if (mode != GM_BRUSH_MAX && mode != GM_BRUSH_MIN && mode != GM_BRUSH_ZERO)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_scalefield_brush: unknown mode");
  gm_status s = set_device(ctx);
  if (s != GM_OK) return s;
  GM_CHECK_CUDA(ctx,
                gm::launch_scale_brush(d_scale, fine_res, bbox_min, cell_size, position, scale, support, global_scale,
                                       (int)mode, (cudaStream_t)stream, &ctx->kc),
                "gm_scalefield_brush");
  return GM_OK;
}

// ------------------------------------------------------------------ a4

int64_t gm_pyramid_texels(int32_t res) {
  if (!pow2(res)) return -1;
  return (int64_t)gm::pyramid_texels(res);
}

gm_status gm_pyramid_build(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_grid, const int8_t* d_scale,
                           int32_t uniform_radius, uint64_t* d_pyramid, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!d_grid || !d_pyramid) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_pyramid_build: NULL buffer");
  if ((s = set_device(ctx)) != GM_OK) return s;
  GM_CHECK_CUDA(ctx, gm::launch_pyramid(d_grid, d_scale, uniform_radius, desc->res, d_pyramid, (cudaStream_t)stream,
                                        &ctx->kc),
                "gm_pyramid_build");
  return GM_OK;
}

// ------------------------------------------------------------------ a5..a11

static gm_status close_impl(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_input, const int8_t* d_scale,
                            int32_t uniform_radius, int mode, int se, uint8_t* d_closing, uint8_t* d_dilation,
                            uint8_t* d_contour, cudaStream_t st, bool xpass_done = false, bool ypass_done = false,
                            int rmax_known = 0, bool zpass_done = false, const gm::RotCubeArgs* rotcube = nullptr) {
  gm_status s;
  const int res = desc->res;
  const int64_t fine = (int64_t)8 * res * res * res;
  if ((s = ensure(ctx, (void**)&ctx->ws, ctx->ws_bytes, gm::close_workspace_bytes(res), "closing workspace")) != GM_OK)
    return s;
  gm::CloseArgs a;
  a.res = res;
  for (int i = 0; i < 3; i++) a.data_res[i] = desc->data_res[i];
  a.X = d_input;
  a.R = d_scale;
  a.uniform_r = uniform_radius;
  a.mode = mode;
  a.se = se;
  a.C_out = d_closing;
  a.D_out = d_dilation;
  a.S_out = d_contour;
  a.workspace = ctx->ws;
  a.num_sms = ctx->num_sms;
  a.rmap_in = d_scale ? ctx->rmap : nullptr;
  a.xpass_done = xpass_done;
  a.ypass_done = ypass_done;
  a.zpass_done = zpass_done;
  int rmax;
  if (d_scale && rmax_known > 0) {
    rmax = rmax_known;  // ctx->rmap and the bound built by the caller (the slab upload of gm_update)
  } else if (d_scale) {
    // the radius bound and the per-tile radius map in one pass over the
    // field, on a side stream; the sphere dilation's x pass (it reads only
    // the grid, saturated for any radius) runs meanwhile on `st`
    if ((s = ensure(ctx, (void**)&ctx->rmap, ctx->rmap_bytes, (size_t)fine / 4096 + 16, "radius map")) != GM_OK)
      return s;
    a.rmap_in = ctx->rmap;
    if (!ctx->copy_st) {
      GM_CHECK_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_st, cudaStreamNonBlocking), "copy stream");
      GM_CHECK_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming), "copy event");
      GM_CHECK_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_geom, cudaEventDisableTiming), "geometry event");
    }
    const bool overlap = se == 0 && !xpass_done && !rotcube;
    cudaStream_t rs = overlap ? ctx->copy_st : st;
    if (overlap) {
      GM_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev_copy, st), "radius bound");
      GM_CHECK_CUDA(ctx, cudaStreamWaitEvent(rs, ctx->ev_copy, 0), "radius bound");
    }
    GM_CHECK_CUDA(ctx, gm::launch_radius_map_dense(d_scale, 2 * res, 2 * res, 2 * res, ctx->rmap, ctx->d_int, rs,
                                                   &ctx->kc),
                  "radius bound");
    if (overlap) {
      // (queued before the read-back below, which blocks the host)
      GM_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev_copy, rs), "radius bound");
      GM_CHECK_CUDA(ctx, gm::launch_close_xpass(a, st, &ctx->kc), "gm_close");
      a.xpass_done = true;
      GM_CHECK_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_copy, 0), "radius bound");
    }
    int h = 0;
    GM_CHECK_CUDA(ctx, cudaMemcpyAsync(&h, ctx->d_int, sizeof(int), cudaMemcpyDeviceToHost, rs), "radius bound");
    GM_CHECK_CUDA(ctx, cudaStreamSynchronize(rs), "radius bound");
    rmax = h < 2 ? 2 : h;
  } else {
    rmax = gm::clamp_radius(uniform_radius);
  }
  a.rmax = rmax;
  if (rotcube) {
    // the rotated-cube dilation into the closing's D, its scratch in the
    // part of the workspace that the erosion writes first
    gm::RotCubeArgs r = *rotcube;
    size_t have = 0;
    r.D = gm::close_ws_dilation(a);
    r.scratch = gm::close_ws_scratch(a, &have);
    r.E = gm::close_ws_field(a);
    r.edt_workspace = ctx->ws;
    r.rmax = rmax;
    r.num_sms = ctx->num_sms;
    if (have < gm::rotcube_scratch_bytes(res)) return fail(ctx, GM_ERR_CUDA, "gm_close_rotcube: workspace too small");
    GM_CHECK_CUDA(ctx, gm::launch_rotcube_dilation(r, st, &ctx->kc), "gm_close_rotcube");
    a.dilation_done = true;
  }
  GM_CHECK_CUDA(ctx, gm::launch_close(a, st, &ctx->kc), "gm_close");
  return GM_OK;
}

gm_status gm_close(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_input, const int8_t* d_scale,
                   int32_t uniform_radius, gm_mode mode, gm_se se, uint8_t* d_closing, uint8_t* d_dilation,
                   uint8_t* d_contour, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!d_input || !d_closing) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close: NULL input or output");
  if (!aligned16(d_input) || (d_scale && !aligned16(d_scale)))
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close: device buffers must be 16-byte aligned");
  if (mode != GM_REF && mode != GM_EXACT) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close: unknown mode");
  if (se != GM_SE_SPHERE && se != GM_SE_CUBE) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close: unknown se");
  if ((s = set_device(ctx)) != GM_OK) return s;
  return close_impl(ctx, desc, d_input, d_scale, uniform_radius, (int)mode, (int)se, d_closing, d_dilation, d_contour,
                    (cudaStream_t)stream);
}

gm_status gm_close_rotcube(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_input, const int8_t* d_scale,
                           int32_t uniform_radius, const float* d_quats, int32_t quat_res, gm_mode mode,
                           uint8_t* d_closing, uint8_t* d_dilation, uint8_t* d_contour, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!d_input || !d_closing || !d_quats)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_rotcube: NULL input, quaternion field or output");
  if (!aligned16(d_input) || (d_scale && !aligned16(d_scale)) || !aligned16(d_quats))
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_rotcube: device buffers must be 16-byte aligned");
  if (quat_res < 1 || quat_res > 1024)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_rotcube: quat_res must lie in [1, 1024]");
  if (mode != GM_REF && mode != GM_EXACT) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_rotcube: unknown mode");
  if ((s = set_device(ctx)) != GM_OK) return s;
  gm::RotCubeArgs r;
  r.res = desc->res;
  for (int i = 0; i < 3; i++) r.data_res[i] = desc->data_res[i];
  r.X = d_input;
  r.R = d_scale;
  r.uniform_r = uniform_radius;
  r.Q = d_quats;
  r.qres = quat_res;
  r.mode = (int)mode;
  return close_impl(ctx, desc, d_input, d_scale, uniform_radius, (int)mode, GM_SE_CUBE, d_closing, d_dilation,
                    d_contour, (cudaStream_t)stream, false, false, 0, false, &r);
}

gm_status gm_contour(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_grid, uint8_t* d_out, gm_mode mode,
                     void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!d_grid || !d_out || !aligned16(d_grid) || !aligned16(d_out))
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_contour: NULL or misaligned buffer");
  if (mode != GM_REF && mode != GM_EXACT) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_contour: unknown mode");
  if ((s = set_device(ctx)) != GM_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t cells = (size_t)desc->res * desc->res * desc->res;
  uint8_t* dst = d_out;
  if (d_out == d_grid) {  // the tagger reads neighbours: write to scratch, then copy back
    if ((s = ensure(ctx, (void**)&ctx->vox, ctx->vox_bytes, cells, "contour scratch")) != GM_OK) return s;
    dst = ctx->vox;
  }
  GM_CHECK_CUDA(ctx, gm::launch_contour(d_grid, dst, desc->res, mode == GM_EXACT ? 1 : 0, st, &ctx->kc), "gm_contour");
  if (dst != d_out) GM_CHECK_CUDA(ctx, cudaMemcpyAsync(d_out, dst, cells, cudaMemcpyDeviceToDevice, st), "gm_contour");
  return GM_OK;
}

// ------------------------------------------------------------------ box grids

static gm_status check_box(gm_ctx* ctx, const gm_box_desc* b) {
  if (!b) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "box descriptor is NULL");
  for (int a = 0; a < 3; a++) {
    if (b->dims[a] < 16 || b->dims[a] % 16 != 0 || b->dims[a] > 2048)
      return fail(ctx, GM_ERR_INVALID_ARGUMENT, "box dims must be multiples of 16 in [16, 2048]");
    if (b->data_res[a] < 0 || b->data_res[a] > b->dims[a])
      return fail(ctx, GM_ERR_INVALID_ARGUMENT, "data_res must lie in [0, dims]");
  }
  if (!(b->cell_size > 0.f)) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "cell_size must be positive");
  return GM_OK;
}

static gm_status close_box_impl(gm_ctx* ctx, const gm_box_desc* box, const uint8_t* d_input, const int8_t* d_scale,
                                int32_t uniform_radius, gm_mode mode, gm_se se, const int32_t* roi_lo,
                                const int32_t* roi_hi, uint8_t* d_closing, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_box(ctx, box);
  if (s != GM_OK) return s;
  if (!d_input || !d_closing) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_box: NULL input or output");
  if (!aligned16(d_input) || (d_scale && !aligned16(d_scale)))
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_box: device buffers must be 16-byte aligned");
  if (mode != GM_REF && mode != GM_EXACT) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_box: unknown mode");
  if (se != GM_SE_SPHERE && se != GM_SE_CUBE) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_box: unknown se");
  if ((s = set_device(ctx)) != GM_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const int rx = box->dims[0], ry = box->dims[1], rz = box->dims[2];
  int rmax;
  if (d_scale) {
    GM_CHECK_CUDA(ctx, gm::launch_rmax(d_scale, (int64_t)8 * rx * ry * rz, ctx->d_int, ctx->num_sms, st, &ctx->kc),
                  "radius bound");
    int h = 0;
    GM_CHECK_CUDA(ctx, cudaMemcpyAsync(&h, ctx->d_int, sizeof(int), cudaMemcpyDeviceToHost, st), "radius bound");
    GM_CHECK_CUDA(ctx, cudaStreamSynchronize(st), "radius bound");
    rmax = h;
  } else {
    rmax = gm::clamp_radius(uniform_radius);
  }
  if ((s = ensure(ctx, (void**)&ctx->ws, ctx->ws_bytes, gm::close_workspace_bytes_box(rx, ry, rz),
                  "closing workspace")) != GM_OK)
    return s;
  gm::CloseArgs a;
  a.res = 0;
  a.dims[0] = rx;
  a.dims[1] = ry;
  a.dims[2] = rz;
  for (int i = 0; i < 3; i++) a.data_res[i] = box->data_res[i];
  a.X = d_input;
  a.R = d_scale;
  a.uniform_r = uniform_radius;
  a.rmax = rmax;
  a.mode = (int)mode;
  a.se = (int)se;
  a.C_out = d_closing;
  a.D_out = nullptr;
  a.S_out = nullptr;
  a.workspace = ctx->ws;
  a.num_sms = ctx->num_sms;
  if (roi_lo && roi_hi)
    for (int k = 0; k < 3; k++) {
      a.roi_lo[k] = roi_lo[k];
      a.roi_hi[k] = roi_hi[k];
    }
  GM_CHECK_CUDA(ctx, gm::launch_close(a, st, &ctx->kc), "gm_close_box");
  return GM_OK;
}

gm_status gm_close_box(gm_ctx* ctx, const gm_box_desc* box, const uint8_t* d_input, const int8_t* d_scale,
                       int32_t uniform_radius, gm_mode mode, gm_se se, uint8_t* d_closing, void* stream) {
  return close_box_impl(ctx, box, d_input, d_scale, uniform_radius, mode, se, nullptr, nullptr, d_closing, stream);
}

gm_status gm_close_box_region(gm_ctx* ctx, const gm_box_desc* box, const uint8_t* d_input, const int8_t* d_scale,
                              int32_t uniform_radius, gm_mode mode, gm_se se, const int32_t roi_lo[3],
                              const int32_t roi_hi[3], uint8_t* d_closing, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  if (!roi_lo || !roi_hi) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_box_region: NULL region");
  for (int k = 0; k < 3; k++)
    if (roi_lo[k] < 0 || roi_hi[k] <= roi_lo[k] || (box && roi_hi[k] > box->dims[k]))
      return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_close_box_region: empty region or region outside the box");
  return close_box_impl(ctx, box, d_input, d_scale, uniform_radius, mode, se, roi_lo, roi_hi, d_closing, stream);
}

gm_status gm_mesh_box(gm_ctx* ctx, const gm_box_desc* box, const uint8_t* d_closing, const gm_mesh_window* win,
                      int32_t bilateral_iters, gm_mesh_view* out, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_box(ctx, box);
  if (s != GM_OK) return s;
  if (!d_closing || !out || bilateral_iters < 0)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_mesh_box: NULL buffer or negative iteration count");
  if (!aligned16(d_closing)) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_mesh_box: the grid must be 16-byte aligned");
  if (win) {
    if (win->global_res < 1) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_mesh_box: global_res must be positive");
    for (int a = 0; a < 3; a++)
      if (win->emit_lo[a] < 0 || win->emit_hi[a] > box->dims[a] || win->emit_lo[a] > win->emit_hi[a] ||
          win->origin[a] < 0 || win->origin[a] + box->dims[a] > win->global_res)
        return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_mesh_box: window outside the box or the global grid");
  }
  if ((s = set_device(ctx)) != GM_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  gm::MeshArgs a;
  a.res = 0;
  for (int k = 0; k < 3; k++) a.dims[k] = box->dims[k];
  a.C = d_closing;
  for (int i = 0; i < 3; i++) a.bbox_min[i] = box->bbox_min[i];
  a.cell_size = box->cell_size;
  a.isovalue = 0.95f;  // GMorpho.cu:6922
  a.bilateral_iters = bilateral_iters;
  a.num_sms = ctx->num_sms;
  if (win) {
    a.gres = win->global_res;
    for (int k = 0; k < 3; k++) {
      a.off[k] = win->origin[k];
      a.emit_lo[k] = win->emit_lo[k];
      a.emit_hi[k] = win->emit_hi[k];
      a.tag_lo[k] = win->emit_lo[k];
      a.tag_hi[k] = win->emit_hi[k] + 1 < box->dims[k] ? win->emit_hi[k] + 1 : box->dims[k];
    }
    a.zero_isolated = 1;
  }
  int64_t nv = 0, nt = 0;
  ctx->has_mesh = false;
  GM_CHECK_CUDA(ctx, gm::mesh_count(a, ctx->mesh, st, &ctx->kc, &nv, &nt), "gm_mesh_box (count)");
  if (nv > 0xfffffff0LL || nt > 0x7ffffff0LL)
    return fail(ctx, GM_ERR_CAPACITY, "gm_mesh_box: mesh exceeds 32-bit vertex/triangle indexing");
  GM_CHECK_CUDA(ctx, gm::mesh_emit(a, ctx->mesh, nv, nt, st, &ctx->kc), "gm_mesh_box (emit)");
  ctx->nv = nv;
  ctx->nt = nt;
  ctx->has_mesh = true;
  out->vertices = ctx->mesh.V;
  out->normals = ctx->mesh.N;
  out->triangles = ctx->mesh.T;
  out->num_vertices = nv;
  out->num_triangles = nt;
  return GM_OK;
}

// ------------------------------------------------------------------ a12..a16

static gm_status mesh_impl(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_closing, int iters,
                           cudaStream_t st, cudaEvent_t geometry_done = nullptr) {
  gm::MeshArgs a;
  a.res = desc->res;
  a.C = d_closing;
  for (int i = 0; i < 3; i++) a.bbox_min[i] = desc->bbox_min[i];
  a.cell_size = desc->cell_size;
  a.isovalue = 0.95f;  // GMorpho.cu:6922
  a.bilateral_iters = iters;
  a.num_sms = ctx->num_sms;
  a.geometry_done = geometry_done;
  int64_t nv = 0, nt = 0;
  ctx->has_mesh = false;
  GM_CHECK_CUDA(ctx, gm::mesh_count(a, ctx->mesh, st, &ctx->kc, &nv, &nt), "gm_mesh (count)");
  if (nv > 0xfffffff0LL || nt > 0x7ffffff0LL)
    return fail(ctx, GM_ERR_CAPACITY, "gm_mesh: mesh exceeds 32-bit vertex/triangle indexing");
  GM_CHECK_CUDA(ctx, gm::mesh_emit(a, ctx->mesh, nv, nt, st, &ctx->kc), "gm_mesh (emit)");
  ctx->nv = nv;
  ctx->nt = nt;
  ctx->has_mesh = true;
  return GM_OK;
}

gm_status gm_mesh(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_closing, int32_t bilateral_iters,
                  gm_mesh_view* out, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!d_closing || !out || bilateral_iters < 0)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_mesh: NULL buffer or negative iteration count");
  if (!aligned16(d_closing)) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_mesh: the grid must be 16-byte aligned");
  if ((s = set_device(ctx)) != GM_OK) return s;
  if ((s = mesh_impl(ctx, desc, d_closing, bilateral_iters, (cudaStream_t)stream)) != GM_OK) return s;
  out->vertices = ctx->mesh.V;
  out->normals = ctx->mesh.N;
  out->triangles = ctx->mesh.T;
  out->num_vertices = ctx->nv;
  out->num_triangles = ctx->nt;
  return GM_OK;
}

// ------------------------------------------------------------------ a17

// Host-buffer update.  The input grid goes up first and the dilation's x
// pass (which reads only the grid) runs while the radius field is still
// being copied on a second stream; with host mesh buffers, the vertices and
// triangles come down on that stream while the normals are filtered.
static gm_status update_impl(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* h_input, const int8_t* h_scale,
                             float global_scale, const gm_update_opts* opts, float* h_V, float* h_N, uint32_t* h_T,
                             int64_t v_cap, int64_t t_cap, int64_t* num_vertices, int64_t* num_triangles,
                             cudaStream_t st) {
  gm_status s;
  const int res = desc->res;
  const size_t cells = (size_t)res * res * res;
  const int asym = opts ? opts->use_asymmetric_closing : 0;
  const int bil = opts ? opts->bilateral_filtering : 1;
  const int mode = opts ? opts->mode : GM_REF;
  if (!ctx->copy_st) {
    GM_CHECK_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_st, cudaStreamNonBlocking), "copy stream");
    GM_CHECK_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming), "copy event");
    GM_CHECK_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_geom, cudaEventDisableTiming), "geometry event");
  }
  if ((s = ensure(ctx, (void**)&ctx->d_X, ctx->X_bytes, cells, "input grid")) != GM_OK) return s;
  if ((s = ensure(ctx, (void**)&ctx->d_C, ctx->C_bytes, cells, "closing grid")) != GM_OK) return s;
  if (h_scale && (s = ensure(ctx, (void**)&ctx->d_R, ctx->R_bytes, 8 * cells, "scale grid")) != GM_OK) return s;
  // uniform radius in fine voxels: floor(global_scale / (cell_size / 2))
  // (GMorpho/ScaleField.cu:143-146 with cell_size_sf = cell_size / 2)
  const float gate = std::floor(2.f * global_scale / desc->cell_size);
  const int uniform = (int)std::floor(global_scale / (0.5f * desc->cell_size));
  const bool morph = gate > 1.f;
  // The radius field arrives in z slabs (sphere closings): each slab's
  // radius map, and the dilation's y pass over a slab once the bounds of the
  // slabs within 128 fine voxels of it are known, run while later slabs are
  // still being copied.
  const int slab_cells = res / gm_ctx::kSlabs;
  const bool slabs = h_scale && morph && !asym && slab_cells % 8 == 0;
  if (slabs && !ctx->h_slab) {
    GM_CHECK_CUDA(ctx, cudaMallocHost(&ctx->h_slab, gm_ctx::kSlabs * sizeof(int)), "slab bounds");
    for (int k = 0; k < gm_ctx::kSlabs; k++) {
      GM_CHECK_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_slab[k], cudaEventDisableTiming), "slab event");
      GM_CHECK_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_max[k], cudaEventDisableTiming), "slab event");
    }
  }
  // the radius field's upload waits only for the work already on the stream
  // (earlier uses of the buffer), then runs beside the grid's upload and x pass
  // (the grid is issued first: copies of one direction are served in order)
  GM_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev_copy, st), "gm_update");
  GM_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->d_X, h_input, cells, cudaMemcpyHostToDevice, st), "gm_update H2D");
  if (h_scale) {
    GM_CHECK_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_st, ctx->ev_copy, 0), "gm_update");
    if (slabs) {
      const size_t slab_bytes = 8 * cells / gm_ctx::kSlabs;
      for (int k = 0; k < gm_ctx::kSlabs; k++) {
        GM_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->d_R + k * slab_bytes, h_scale + k * slab_bytes, slab_bytes,
                                           cudaMemcpyHostToDevice, ctx->copy_st),
                      "gm_update H2D");
        GM_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev_slab[k], ctx->copy_st), "gm_update");
      }
    } else {
      GM_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->d_R, h_scale, 8 * cells, cudaMemcpyHostToDevice, ctx->copy_st),
                    "gm_update H2D");
    }
    GM_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev_copy, ctx->copy_st), "gm_update");
  }
  bool xpass = false;
  if (morph) {
    if ((s = ensure(ctx, (void**)&ctx->ws, ctx->ws_bytes, gm::close_workspace_bytes(res), "closing workspace")) !=
        GM_OK)
      return s;
    gm::CloseArgs a;
    a.res = res;
    a.X = ctx->d_X;
    a.workspace = ctx->ws;
    GM_CHECK_CUDA(ctx, gm::launch_close_xpass(a, st, &ctx->kc), "gm_update x pass");
    xpass = true;
  }
  const int8_t* d_scale = nullptr;
  int rmax_known = 0;
  bool zpass = false;
  if (slabs) {
    const int N = 2 * res, mb = N / 16;
    const int slab_fine = 2 * slab_cells;
    const size_t slab_bytes = (size_t)N * N * slab_fine;
    const size_t slab_blocks = (size_t)mb * mb * (slab_fine / 16);
    const int reach = (128 + slab_fine - 1) / slab_fine;  // slabs within 128 fine voxels
    if ((s = ensure(ctx, (void**)&ctx->rmap, ctx->rmap_bytes, 8 * cells / 4096 + 16, "radius map")) != GM_OK) return s;
    gm::CloseArgs a;
    a.res = res;
    a.X = ctx->d_X;
    a.workspace = ctx->ws;
    a.se = 0;
    a.rmap_in = ctx->rmap;
    const bool zslabs = slab_cells % 32 == 0;  // whole z-pass output tiles per slab
    a.mode = mode;
    a.R = ctx->d_R;
    int bound[gm_ctx::kSlabs];
    int next = 0, znext = 0;  // next slabs whose y / z pass is due
    for (int k = 0; k < gm_ctx::kSlabs; k++) {
      GM_CHECK_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_slab[k], 0), "gm_update");
      GM_CHECK_CUDA(ctx, gm::launch_radius_map_dense(ctx->d_R + k * slab_bytes, N, N, slab_fine,
                                                     ctx->rmap + k * slab_blocks, ctx->d_int + k, st, &ctx->kc),
                    "radius bound");
      GM_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->h_slab + k, ctx->d_int + k, sizeof(int), cudaMemcpyDeviceToHost, st),
                    "radius bound");
      GM_CHECK_CUDA(ctx, cudaEventRecord(ctx->ev_max[k], st), "radius bound");
      // y passes whose neighbouring bounds are all known now
      const int upto = k == gm_ctx::kSlabs - 1 ? gm_ctx::kSlabs : k + 1 - reach;
      if (next < upto) GM_CHECK_CUDA(ctx, cudaEventSynchronize(ctx->ev_max[k]), "radius bound");
      for (; next < upto; next++) {
        int rb = 2;
        for (int j = std::max(0, next - reach); j <= std::min(gm_ctx::kSlabs - 1, next + reach); j++)
          rb = std::max(rb, ctx->h_slab[j]);
        bound[next] = rb;
        GM_CHECK_CUDA(ctx, gm::launch_close_ypass(a, next * slab_cells, (next + 1) * slab_cells, rb, st, &ctx->kc),
                      "gm_update y pass");
        // z passes whose window's y passes are all issued now
        const int zupto = next == gm_ctx::kSlabs - 1 ? gm_ctx::kSlabs : next + 1 - reach;
        for (; zslabs && znext < zupto; znext++)
          GM_CHECK_CUDA(ctx, gm::launch_close_zpass(a, znext * slab_cells, (znext + 1) * slab_cells, bound[znext],
                                                    st, &ctx->kc),
                        "gm_update z pass");
      }
    }
    zpass = zslabs;
    for (int k = 0; k < gm_ctx::kSlabs; k++) rmax_known = std::max(rmax_known, ctx->h_slab[k]);
    rmax_known = std::max(rmax_known, 2);
  }
  if (h_scale) {
    GM_CHECK_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_copy, 0), "gm_update");
    d_scale = ctx->d_R;
  }
  if (morph) {
    s = close_impl(ctx, desc, ctx->d_X, d_scale, uniform, mode, asym ? GM_SE_CUBE : GM_SE_SPHERE, ctx->d_C, nullptr,
                   nullptr, st, xpass, slabs, rmax_known, zpass);
    if (s != GM_OK) return s;
  } else {
    GM_CHECK_CUDA(ctx, cudaMemcpyAsync(ctx->d_C, ctx->d_X, cells, cudaMemcpyDeviceToDevice, st), "gm_update copy");
  }
  const int iters = bil ? (asym ? 200 : 20) : 0;  // GMorpho.cu:7808-7811
  const bool to_host = h_V != nullptr || h_N != nullptr || h_T != nullptr;
  if ((s = mesh_impl(ctx, desc, ctx->d_C, iters, st, to_host ? ctx->ev_geom : nullptr)) != GM_OK) return s;
  if (num_vertices) *num_vertices = ctx->nv;
  if (num_triangles) *num_triangles = ctx->nt;
  if (!to_host) return GM_OK;
  if (ctx->nv > v_cap || ctx->nt > t_cap) {
    GM_CHECK_CUDA(ctx, cudaStreamSynchronize(st), "gm_update_to_host");
    return fail(ctx, GM_ERR_CAPACITY, "gm_update_to_host: host mesh buffers too small (mesh kept on the device)");
  }
  // geometry down on the copy stream while the normals are filtered
  GM_CHECK_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_st, ctx->ev_geom, 0), "gm_update_to_host");
  if (h_V && ctx->nv)
    GM_CHECK_CUDA(ctx, cudaMemcpyAsync(h_V, ctx->mesh.V, 12 * (size_t)ctx->nv, cudaMemcpyDeviceToHost, ctx->copy_st),
                  "D2H");
  if (h_T && ctx->nt)
    GM_CHECK_CUDA(ctx, cudaMemcpyAsync(h_T, ctx->mesh.T, 12 * (size_t)ctx->nt, cudaMemcpyDeviceToHost, ctx->copy_st),
                  "D2H");
  if (h_N && ctx->nv)
    GM_CHECK_CUDA(ctx, cudaMemcpyAsync(h_N, ctx->mesh.N, 12 * (size_t)ctx->nv, cudaMemcpyDeviceToHost, st), "D2H");
  GM_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->copy_st), "gm_update_to_host");
  GM_CHECK_CUDA(ctx, cudaStreamSynchronize(st), "gm_update_to_host");
  return GM_OK;
}

gm_status gm_update(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* h_input, const int8_t* h_scale,
                    float global_scale, const gm_update_opts* opts, int64_t* num_vertices, int64_t* num_triangles,
                    void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!h_input) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_update: NULL input grid");
  if ((s = set_device(ctx)) != GM_OK) return s;
  return update_impl(ctx, desc, h_input, h_scale, global_scale, opts, nullptr, nullptr, nullptr, 0, 0, num_vertices,
                     num_triangles, (cudaStream_t)stream);
}

gm_status gm_update_to_host(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* h_input, const int8_t* h_scale,
                            float global_scale, const gm_update_opts* opts, float* h_V, float* h_N, uint32_t* h_T,
                            int64_t vertex_capacity, int64_t triangle_capacity, int64_t* num_vertices,
                            int64_t* num_triangles, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!h_input || (!h_V && !h_N && !h_T) || vertex_capacity < 0 || triangle_capacity < 0)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_update_to_host: NULL input or no output buffer");
  if ((s = set_device(ctx)) != GM_OK) return s;
  return update_impl(ctx, desc, h_input, h_scale, global_scale, opts, h_V, h_N, h_T, vertex_capacity,
                     triangle_capacity, num_vertices, num_triangles, (cudaStream_t)stream);
}

gm_status gm_mesh_download(gm_ctx* ctx, float* h_V, float* h_N, uint32_t* h_T, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  if (!ctx->has_mesh) return fail(ctx, GM_ERR_NOT_READY, "gm_mesh_download: no mesh on this context");
  gm_status s = set_device(ctx);
  if (s != GM_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  if (h_V && ctx->nv)
    GM_CHECK_CUDA(ctx, cudaMemcpyAsync(h_V, ctx->mesh.V, 12 * (size_t)ctx->nv, cudaMemcpyDeviceToHost, st), "D2H");
  if (h_N && ctx->nv)
    GM_CHECK_CUDA(ctx, cudaMemcpyAsync(h_N, ctx->mesh.N, 12 * (size_t)ctx->nv, cudaMemcpyDeviceToHost, st), "D2H");
  if (h_T && ctx->nt)
    GM_CHECK_CUDA(ctx, cudaMemcpyAsync(h_T, ctx->mesh.T, 12 * (size_t)ctx->nt, cudaMemcpyDeviceToHost, st), "D2H");
  GM_CHECK_CUDA(ctx, cudaStreamSynchronize(st), "gm_mesh_download");
  return GM_OK;
}

// ------------------------------------------------------------------ batch

gm_status gm_batch_close_mesh(gm_ctx* ctx, int32_t n, const gm_batch_item* items, gm_mode mode, gm_se se,
                              int32_t bilateral_iters, int32_t lanes, gm_mesh_view* meshes, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  if (n < 0 || (n > 0 && !items) || bilateral_iters < 0 || lanes < GM_BATCH_GROUPED || lanes > 64)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_batch_close_mesh: bad argument");
  if (mode != GM_REF && mode != GM_EXACT) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_batch_close_mesh: mode");
  if (se != GM_SE_SPHERE && se != GM_SE_CUBE) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_batch_close_mesh: se");
  for (int i = 0; i < n; i++) {
    gm_status s = check_desc(ctx, &items[i].desc);
    if (s != GM_OK) return s;
    if (!items[i].d_input || !items[i].d_closing || !aligned16(items[i].d_input) ||
        !aligned16(items[i].d_closing) || (items[i].d_scale && !aligned16(items[i].d_scale)))
      return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_batch_close_mesh: item " + std::to_string(i));
  }
  if (n == 0) return GM_OK;
  gm_status s = set_device(ctx);
  if (s != GM_OK) return s;
  ctx->has_mesh = false;
  const cudaError_t e = gm::batch_run(&ctx->batch, n, items, (int)mode, (int)se, bilateral_iters, lanes, meshes,
                                      ctx->num_sms, (cudaStream_t)stream, &ctx->kc);
  if (e == cudaErrorNotSupported)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_batch_close_mesh: the grouped form needs radius bounds <= 91");
  GM_CHECK_CUDA(ctx, e, "gm_batch_close_mesh");
  return GM_OK;
}

int32_t gm_batch_lanes(gm_ctx* ctx) { return ctx ? gm::batch_lanes_tuned(ctx->batch) : 0; }

gm_status gm_batch_inject_alloc_failures(gm_ctx* ctx, int32_t count) {
  if (!ctx || count < 0) return GM_ERR_INVALID_ARGUMENT;
  gm::batch_inject_alloc_failures(&ctx->batch, count);
  return GM_OK;
}

// ------------------------------------------------------------------ a18

struct gm_bvh {
  void* dev = nullptr;
  int64_t n = 0;
  int device = 0;
};

static gm_status bvh_build_impl(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_sites, gm_bvh** out,
                                cudaStream_t st) {
  const int res = desc->res;
  const size_t nb = (size_t)res * res * res / 4096;
  gm_status s;
  if ((s = ensure(ctx, (void**)&ctx->vox, ctx->vox_bytes, sizeof(uint32_t) * (nb + 1), "bvh scratch")) != GM_OK)
    return s;
  void* h = nullptr;
  int n = 0;
  GM_CHECK_CUDA(ctx, gm::bvh_build(d_sites, res, &h, reinterpret_cast<uint32_t*>(ctx->vox), &n, st, &ctx->kc),
                "gm_bvh_build");
  gm_bvh* b = new gm_bvh();
  b->dev = h;
  b->n = n;
  b->device = ctx->device;
  *out = b;
  return GM_OK;
}

gm_status gm_bvh_build(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_sites, gm_bvh** out,
                       int64_t* num_leaves, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!d_sites || !out) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_bvh_build: NULL argument");
  if ((s = set_device(ctx)) != GM_OK) return s;
  if ((s = bvh_build_impl(ctx, desc, d_sites, out, (cudaStream_t)stream)) != GM_OK) return s;
  if (num_leaves) *num_leaves = (*out)->n;
  return GM_OK;
}

gm_status gm_bvh_destroy(gm_bvh* bvh) {
  if (!bvh) return GM_ERR_INVALID_ARGUMENT;
  cudaSetDevice(bvh->device);
  gm::bvh_free(bvh->dev);
  delete bvh;
  return GM_OK;
}

gm_status gm_bvh_query(gm_ctx* ctx, const gm_bvh* bvh, const int32_t* d_points2, int64_t n, int32_t radius,
                       uint8_t* d_hits, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  if (!bvh || (n > 0 && (!d_points2 || !d_hits)) || n < 0 || radius < 0)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_bvh_query: bad argument");
  gm_status s = set_device(ctx);
  if (s != GM_OK) return s;
  GM_CHECK_CUDA(ctx, gm::bvh_query(bvh->dev, d_points2, n, radius, d_hits, (cudaStream_t)stream, &ctx->kc),
                "gm_bvh_query");
  return GM_OK;
}

gm_status gm_bvh_leaves(gm_ctx* ctx, const gm_bvh* bvh, uint64_t* d_keys, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  if (!bvh || !d_keys) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_bvh_leaves: NULL argument");
  gm_status s = set_device(ctx);
  if (s != GM_OK) return s;
  GM_CHECK_CUDA(ctx, gm::bvh_keys(bvh->dev, d_keys, (cudaStream_t)stream), "gm_bvh_leaves");
  return GM_OK;
}

gm_status gm_erode_bvh(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_input, const uint8_t* d_dilation,
                       int32_t radius, uint8_t* d_closing, void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  gm_status s = check_desc(ctx, desc);
  if (s != GM_OK) return s;
  if (!d_input || !d_dilation || !d_closing || !aligned16(d_dilation) || radius < 0)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_erode_bvh: bad argument");
  if ((s = set_device(ctx)) != GM_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t cells = (size_t)desc->res * desc->res * desc->res;
  // contour of the dilation into the closing workspace, then its BVH
  if ((s = ensure(ctx, (void**)&ctx->ws, ctx->ws_bytes, gm::close_workspace_bytes(desc->res), "workspace")) != GM_OK)
    return s;
  uint8_t* S = ctx->ws;
  GM_CHECK_CUDA(ctx, gm::launch_contour(d_dilation, S, desc->res, 0, st, &ctx->kc), "gm_erode_bvh contour");
  gm_bvh* b = nullptr;
  if ((s = bvh_build_impl(ctx, desc, S, &b, st)) != GM_OK) return s;
  int* d_over = ctx->d_int + 1;
  const cudaError_t e = gm::bvh_erode(b->dev, d_input, d_dilation, desc->res, desc->data_res, radius, d_closing,
                                      d_over, st, &ctx->kc);
  int over = 0;
  cudaMemcpyAsync(&over, d_over, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  gm_bvh_destroy(b);
  (void)cells;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gm_erode_bvh");
  if (over) return fail(ctx, GM_ERR_CAPACITY, "gm_erode_bvh: traversal stack overflow");
  return GM_OK;
}

// ------------------------------------------------------------------ layout

gm_status gm_layout_zwords_to_packed(gm_ctx* ctx, int32_t res, const uint32_t* d_zwords, uint8_t* d_grid,
                                     void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  if (!pow2(res) || res < 16 || res > 1024 || !d_zwords || !d_grid)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_layout_zwords_to_packed: bad argument");
  gm_status s = set_device(ctx);
  if (s != GM_OK) return s;
  GM_CHECK_CUDA(ctx, gm::launch_layout(res, d_zwords, d_grid, 0, (cudaStream_t)stream, &ctx->kc), "layout");
  return GM_OK;
}

gm_status gm_layout_packed_to_zwords(gm_ctx* ctx, int32_t res, const uint8_t* d_grid, uint32_t* d_zwords,
                                     void* stream) {
  if (!ctx) return GM_ERR_INVALID_ARGUMENT;
  if (!pow2(res) || res < 16 || res > 1024 || !d_zwords || !d_grid)
    return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_layout_packed_to_zwords: bad argument");
  gm_status s = set_device(ctx);
  if (s != GM_OK) return s;
  GM_CHECK_CUDA(ctx, gm::launch_layout(res, d_zwords, const_cast<uint8_t*>(d_grid), 1, (cudaStream_t)stream, &ctx->kc),
                "layout");
  return GM_OK;
}

// ------------------------------------------------------------------ frame field

}  // extern "C"

struct gm_frame_field {
  gm_ctx* ctx = nullptr;
  int res = 0;
  float bbox_min[3] = {0, 0, 0}, bbox_max[3] = {0, 0, 0};
  float cell_size = 0.f;
  struct Point {
    float grid[3];   // floored lattice position
    float twist[3];  // rotation vector (axis * angle)
  };
  std::vector<Point> points;
  gm::FrameFieldGpu gpu;
  bool generated = false;
};

namespace {

constexpr int kMaxHardConstraints = 20;  // max_hc_number_ (GMorpho/FrameField.h, FrameField::FrameField)

// The constraint quaternion (sin(theta/2) v, cos(theta/2)) of a twist:
// theta = |twist| in float, v = twist scaled by 1.f / theta (left as is when
// theta is 0), sine and cosine in double (FrameFieldSparseBiharmonic.cu:
// 487-503; Common/Vec3.h:203-216).
void twist_quat(const float* tw, float* q) {
  const float theta = (float)std::sqrt((double)(tw[0] * tw[0] + tw[1] * tw[1] + tw[2] * tw[2]));
  float v[3] = {tw[0], tw[1], tw[2]};
  if (theta != 0.0f) {
    const float inv = 1.0f / theta;
    for (int i = 0; i < 3; i++) v[i] *= inv;
  }
  const double s = std::sin(0.5 * (double)theta), c = std::cos(0.5 * (double)theta);
  for (int i = 0; i < 3; i++) q[i] = (float)(s * (double)v[i]);
  q[3] = (float)c;
}

}  // namespace

extern "C" {

gm_status gm_frame_field_create(gm_ctx* ctx, const float* bbox_min, const float* bbox_max, int32_t res,
                                gm_frame_field** out) {
  if (!ctx || !bbox_min || !bbox_max || !out) return GM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (res < 2 || res > 256) return fail(ctx, GM_ERR_INVALID_ARGUMENT, "gm_frame_field_create: res must lie in [2, 256]");
  gm_status s;
  if ((s = set_device(ctx)) != GM_OK) return s;
  gm_frame_field* f = new gm_frame_field();
  f->ctx = ctx;
  f->res = res;
  for (int i = 0; i < 3; i++) f->bbox_min[i] = bbox_min[i], f->bbox_max[i] = bbox_max[i];
  // InitSparseBiharmonicSystem (FrameFieldSparseBiharmonic.cu:28-38)
  f->cell_size = std::max(std::fabs(bbox_max[0] - bbox_min[0]),
                          std::max(std::fabs(bbox_max[1] - bbox_min[1]), std::fabs(bbox_max[2] - bbox_min[2]))) /
                 (float)res;
  cudaError_t e = gm::frame_field_alloc(f->gpu, res);
  if (e != cudaSuccess) {
    cudaGetLastError();
    gm::frame_field_free(f->gpu);
    delete f;
    return fail(ctx, e == cudaErrorMemoryAllocation ? GM_ERR_OUT_OF_MEMORY : GM_ERR_CUDA,
                std::string("gm_frame_field_create: ") + cudaGetErrorString(e));
  }
  *out = f;
  return GM_OK;
}

gm_status gm_frame_field_destroy(gm_frame_field* ff) {
  if (!ff) return GM_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ff->ctx->device);
  gm::frame_field_free(ff->gpu);
  delete ff;
  return GM_OK;
}

gm_status gm_frame_field_add_point(gm_frame_field* ff, const float* position, const float* twist) {
  if (!ff || !position || !twist) return GM_ERR_INVALID_ARGUMENT;
  if ((int)ff->points.size() >= kMaxHardConstraints)
    return fail(ff->ctx, GM_ERR_CAPACITY, "gm_frame_field_add_point: at most 20 hard constraints");
  // AddHardConstrainedPoint (FrameField.cu:64-77): lattice position
  // floor((position - bbox_min) * (1 / cell_size))
  gm_frame_field::Point pt;
  const float inv = 1.f / ff->cell_size;
  for (int i = 0; i < 3; i++) {
    pt.grid[i] = std::floor((position[i] - ff->bbox_min[i]) * inv);
    pt.twist[i] = twist[i];
    if (!(pt.grid[i] >= 0.f && pt.grid[i] < (float)ff->res))
      return fail(ff->ctx, GM_ERR_INVALID_ARGUMENT, "gm_frame_field_add_point: position outside the field's box");
  }
  ff->points.push_back(pt);
  return GM_OK;
}

gm_status gm_frame_field_update_point(gm_frame_field* ff, int32_t i, const float* twist) {
  if (!ff || !twist) return GM_ERR_INVALID_ARGUMENT;
  if (i < 0 || i >= (int32_t)ff->points.size())
    return fail(ff->ctx, GM_ERR_INVALID_ARGUMENT, "gm_frame_field_update_point: no such point");
  for (int k = 0; k < 3; k++) ff->points[i].twist[k] = twist[k];
  return GM_OK;
}

int32_t gm_frame_field_num_points(const gm_frame_field* ff) { return ff ? (int32_t)ff->points.size() : -1; }

gm_status gm_frame_field_get_point(const gm_frame_field* ff, int32_t i, float* grid_position, float* twist) {
  if (!ff || i < 0 || i >= (int32_t)ff->points.size()) return GM_ERR_INVALID_ARGUMENT;
  for (int k = 0; k < 3; k++) {
    if (grid_position) grid_position[k] = ff->points[i].grid[k];
    if (twist) twist[k] = ff->points[i].twist[k];
  }
  return GM_OK;
}

gm_status gm_frame_field_generate(gm_frame_field* ff, int32_t* iterations, void* stream) {
  if (!ff) return GM_ERR_INVALID_ARGUMENT;
  gm_ctx* ctx = ff->ctx;
  gm_status s;
  if ((s = set_device(ctx)) != GM_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  if (iterations) *iterations = 0;
  if (ff->points.empty()) {
    // InitQuats writes (0, 1, 0, 0) whatever it is given
    // (FrameFieldSparseBiharmonic.cu:649-671)
    GM_CHECK_CUDA(ctx, gm::frame_field_fill(ff->gpu, 0.f, 1.f, 0.f, 0.f, st, &ctx->kc), "gm_frame_field_generate");
  } else {
    const int n = (int)ff->points.size();
    std::vector<int64_t> nodes(n);
    std::vector<float> rhs(4 * (size_t)n);
    const int64_t r = ff->res;
    for (int c = 0; c < n; c++) {
      const auto& pt = ff->points[c];
      nodes[c] = (int64_t)pt.grid[0] + r * (int64_t)pt.grid[1] + r * r * (int64_t)pt.grid[2];
      twist_quat(pt.twist, &rhs[4 * (size_t)c]);
    }
    int it = 0;
    GM_CHECK_CUDA(ctx, gm::frame_field_solve(ff->gpu, nodes.data(), rhs.data(), n, 1e-10, 400000, &it, st, &ctx->kc),
                  "gm_frame_field_generate");
    if (iterations) *iterations = it;
  }
  ff->generated = true;
  return GM_OK;
}

gm_status gm_frame_field_quats(const gm_frame_field* ff, const float** d_quats, int32_t* res) {
  if (!ff || !d_quats) return GM_ERR_INVALID_ARGUMENT;
  if (!ff->generated) return fail(ff->ctx, GM_ERR_NOT_READY, "gm_frame_field_quats: generate first");
  *d_quats = reinterpret_cast<const float*>(ff->gpu.quats);
  if (res) *res = ff->res;
  return GM_OK;
}

// RotationToTwistCayley (FrameField.cu:228-252): the Cayley transform
// C = (R - I)(R + I)^-1 of the rotation with columns e_x, e_y, e_z gives the
// axis (-C12, C02, -C01), normalised; the angle is
// acos(clamp((trace - 1) / 2)).  In double; R + I singular (half turns)
// is rejected.
gm_status gm_rotation_to_twist(const float* e_x, const float* e_y, const float* e_z, float* twist) {
  if (!e_x || !e_y || !e_z || !twist) return GM_ERR_INVALID_ARGUMENT;
  double R[3][3];
  for (int i = 0; i < 3; i++) R[i][0] = e_x[i], R[i][1] = e_y[i], R[i][2] = e_z[i];
  double P[3][3], M[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      P[i][j] = R[i][j] + (i == j ? 1.0 : 0.0);
      M[i][j] = R[i][j] - (i == j ? 1.0 : 0.0);
    }
  // inverse of P by its adjugate
  double A[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      const int i1 = (j + 1) % 3, i2 = (j + 2) % 3, j1 = (i + 1) % 3, j2 = (i + 2) % 3;
      A[i][j] = P[i1][j1] * P[i2][j2] - P[i1][j2] * P[i2][j1];
    }
  const double det = P[0][0] * A[0][0] + P[0][1] * A[1][0] + P[0][2] * A[2][0];
  if (!(std::fabs(det) > 1e-12)) return GM_ERR_INVALID_ARGUMENT;
  double C[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double t = 0;
      for (int k = 0; k < 3; k++) t += M[i][k] * A[k][j];
      C[i][j] = t / det;
    }
  double ax[3] = {-C[1][2], C[0][2], -C[0][1]};
  const double len = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
  if (len != 0.0)
    for (double& a : ax) a /= len;
  const double cth = (R[0][0] + R[1][1] + R[2][2] - 1.0) / 2.0;
  const double theta = std::acos(std::min(std::max(cth, -1.0), 1.0));
  for (int i = 0; i < 3; i++) twist[i] = (float)(theta * ax[i]);
  return GM_OK;
}

}  // extern "C"
