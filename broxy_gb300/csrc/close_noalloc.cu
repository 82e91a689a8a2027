// close_noalloc.cu — gm_close_noalloc: the closing of gm_close with its
// scratch memory in a fixed-size array that the library itself holds in
// device memory, so that the call allocates nothing.
//
// Who needs it: a host application that owns the whole device memory
// budget and does not let plug-in libraries call cudaMalloc/cudaFree (a
// renderer or DCC host, a process that has already carved up the GPU among
// several engines), or a latency-bound loop that cannot afford the implicit
// device synchronisation of cudaMalloc/cudaFree.  Such a caller still
// passes its own input and output buffers; only the intermediate fields of
// the closing live here.
//
// Limit: the scratch array is kStaticScratchBytes (16 MiB); grids up to
// res = 64 base cells per axis (128^3 fine voxels) fit.  Every GPU that
// loads the library holds this array until the process exits.
#include <cuda_runtime.h>

#include "../../include/gmorpho_gb300.h"
#include "gm_common.cuh"
#include "gm_internal.h"

namespace {

constexpr size_t kStaticScratchBytes = (size_t)16 << 20;
// Layout of the array: the radius bound (one int), the 16^3-block radius
// map of a radius field, then the closing workspace.
constexpr size_t kRmaxSlotBytes = 256;

__device__ __align__(256) uint8_t g_close_scratch[kStaticScratchBytes];

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }
size_t rmap_slot_bytes(int res) { return round256((size_t)8 * res * res * res / 4096 + 16); }

// The array's name is only a host-side stand-in: host code must use the
// device address that cudaGetSymbolAddress gives for the current device and
// context.  It is looked up on every call (the lookup allocates nothing), so
// that a device reset or another context made current on the same device
// never leaves a stale address behind.
cudaError_t scratch_for_current_device(uint8_t** out, int* sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_close_scratch);
  if (e != cudaSuccess) return e;
  int n = 0;
  e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  *out = static_cast<uint8_t*>(p);
  *sms = n;
  return cudaSuccess;
}

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

extern "C" gm_status gm_close_noalloc(const gm_grid_desc* desc, const uint8_t* d_input, const int8_t* d_scale,
                                      int32_t uniform_radius, gm_mode mode, gm_se se, uint8_t* d_closing,
                                      uint8_t* d_dilation, uint8_t* d_contour, void* stream) {
  if (!desc || !pow2(desc->res) || desc->res < 16 || desc->res > 1024) return GM_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; a++)
    if (desc->data_res[a] < 0 || desc->data_res[a] > desc->res) return GM_ERR_INVALID_ARGUMENT;
  if (!d_input || !d_closing || !aligned16(d_input) || (d_scale && !aligned16(d_scale)))
    return GM_ERR_INVALID_ARGUMENT;
  if ((mode != GM_REF && mode != GM_EXACT) || (se != GM_SE_SPHERE && se != GM_SE_CUBE)) return GM_ERR_INVALID_ARGUMENT;
  const int res = desc->res;
  const size_t ws_offset = kRmaxSlotBytes + rmap_slot_bytes(res);
  if (ws_offset + gm::close_workspace_bytes(res) > kStaticScratchBytes) return GM_ERR_CAPACITY;

  cudaStream_t st = (cudaStream_t)stream;
  uint8_t* scratch = nullptr;
  int sms = 0;
  if (scratch_for_current_device(&scratch, &sms) != cudaSuccess) {
    cudaGetLastError();
    return GM_ERR_CUDA;
  }
  gm::CloseArgs a;
  int rmax = gm::clamp_radius(uniform_radius);
  if (d_scale) {
    // One pass over the field gives the tile radius map that the dilation
    // reads and the radius bound; the host needs the bound to size the
    // passes, so this waits for the stream (no stream capture is possible
    // with a radius field).
    int* d_rmax = reinterpret_cast<int*>(scratch);  // cleared by the map's launch
    uint8_t* d_rmap = scratch + kRmaxSlotBytes;
    if (gm::launch_radius_map_dense(d_scale, 2 * res, 2 * res, 2 * res, d_rmap, d_rmax, st, nullptr) != cudaSuccess)
      return GM_ERR_CUDA;
    int h = 0;
    if (cudaMemcpyAsync(&h, d_rmax, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return GM_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return GM_ERR_CUDA;
    rmax = h < 2 ? 2 : h;
    a.rmap_in = d_rmap;
  }
  a.res = res;
  for (int i = 0; i < 3; i++) a.data_res[i] = desc->data_res[i];
  a.X = d_input;
  a.R = d_scale;
  a.uniform_r = uniform_radius;
  a.rmax = rmax;
  a.mode = (int)mode;
  a.se = (int)se;
  a.C_out = d_closing;
  a.D_out = d_dilation;
  a.S_out = d_contour;
  a.workspace = scratch + ws_offset;  // every field is written before it is read
  a.num_sms = sms;
  return gm::launch_close(a, st, nullptr) == cudaSuccess ? GM_OK : GM_ERR_CUDA;
}
