// gmref_shim.h — force-included (nvcc -include) into every translation unit
// of the reference build in oracle/_ref/.  TEST INFRASTRUCTURE ONLY: the
// reference GMorpho is built here as a second, independent oracle; the
// product never links or loads it.
//
// What it adapts, without editing the reference files:
//  * __shfl (removed after CUDA 8) becomes __shfl_sync over the whole warp.
//    Its three uses (GMorpho/GMorpho.cu:5369, 5706, 5833) broadcast lane 0's
//    work-counter value at the bottom of a persistent loop that every
//    non-exited lane of the warp reaches; exited lanes do not take part in
//    a *_sync intrinsic, and lane 0 holds the warp's smallest index, so it is
//    alive whenever any lane is.
//  * Three handles of the voxelizer's class declaration (Voxelizer.h:104-106)
//    are unsigned ints, and GL::Program is only named by pointer in method
//    declarations; the voxelizer itself is not built (stubs.cpp).
//  * Device allocations and texture/surface object creation made by the
//    reference go through checked wrappers: a failure throws before any
//    kernel could use a null pointer or an invalid object.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

// (after the CUDA headers that declare their own __shfl overloads)
#define __shfl(var, lane) __shfl_sync(0xffffffffu, (var), (lane))

typedef unsigned int GLuint;
namespace MorphoGraphics {
namespace GL {
class Program;
}
}  // namespace MorphoGraphics

#ifndef GMREF_NO_WRAP
namespace gmref {
inline void fail(const char* what, cudaError_t e) {
  throw std::runtime_error(std::string("reference build: ") + what + ": " + cudaGetErrorString(e));
}
template <typename T>
inline cudaError_t checked_malloc(T** p, size_t bytes) {
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess || (bytes > 0 && *p == nullptr)) fail("cudaMalloc", e);
  return e;
}
inline cudaError_t checked_mipmap(cudaMipmappedArray_t* a, const cudaChannelFormatDesc* d, cudaExtent x,
                                  unsigned int levels, unsigned int flags = 0) {
  cudaError_t e = cudaMallocMipmappedArray(a, d, x, levels, flags);
  if (e != cudaSuccess || *a == nullptr) fail("cudaMallocMipmappedArray", e);
  return e;
}
inline cudaError_t checked_tex(cudaTextureObject_t* t, const cudaResourceDesc* r, const cudaTextureDesc* d,
                               const cudaResourceViewDesc* v) {
  cudaError_t e = cudaCreateTextureObject(t, r, d, v);
  if (e != cudaSuccess || *t == 0) fail("cudaCreateTextureObject", e);
  return e;
}
inline cudaError_t checked_surf(cudaSurfaceObject_t* s, const cudaResourceDesc* r) {
  cudaError_t e = cudaCreateSurfaceObject(s, r);
  if (e != cudaSuccess || *s == 0) fail("cudaCreateSurfaceObject", e);
  return e;
}
}  // namespace gmref
#define cudaMalloc(p, b) gmref::checked_malloc((p), (b))
#define cudaMallocMipmappedArray(...) gmref::checked_mipmap(__VA_ARGS__)
#define cudaCreateTextureObject(...) gmref::checked_tex(__VA_ARGS__)
#define cudaCreateSurfaceObject(...) gmref::checked_surf(__VA_ARGS__)
#endif
