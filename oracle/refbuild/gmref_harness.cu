// gmref_harness.cu — a C entry point around the reference GMorpho built from
// its own sources (oracle/refbuild/build_ref.py).  TEST INFRASTRUCTURE ONLY:
// the tests use it as a second oracle; the product never links or loads it.
//
// gmref_update runs GMorpho::Update(Mesh&, const ScaleField&, const
// FrameField&) (GMorpho/GMorpho.cu:7775-7817) on a packed input grid and a
// fine radius grid given by the caller, in place of GMorpho::Load
// (GMorpho.cu:7731-7773), whose voxelizer needs OpenGL: the grids, box,
// resolution and cell size that Load takes from the voxelizer are set
// directly, then Load's own allocation steps run (Grid::Init,
// CopyVoxelsFrom, ErodeAllocation, ExtractClosingMeshAllocation).  The
// caller (tests/test_oracle_ref.py) checks beforehand, with the C oracle,
// that the input keeps the reference kernels inside their buffers: the
// persistent erosion kernel's first pass reads 1600 list entries
// (GMorpho.cu:5061-5065, 6674-6688), so its list must hold at least that
// many cells, and the mesh must fit the fixed MAX_* buffers (GMorpho.h:39-41).
#include <cuda_runtime.h>
#include <cuda_profiler_api.h>
#include <omp.h>
#include <stdint.h>
#include <string.h>

#include <cassert>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <queue>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <cusolverSp.h>
#include <cusolverSp_LOWLEVEL_PREVIEW.h>
#include <thrust/device_ptr.h>
#include <thrust/device_vector.h>
#include <thrust/host_vector.h>
#include <thrust/remove.h>
#include <thrust/scan.h>
#include <thrust/sort.h>

// The harness sets GMorpho's private state the way Load does; the reference
// class keeps it private, so this one translation unit (which also compiles
// GMorpho.cu itself) opens the access specifiers.
#define private public
#define protected public
#include <GMorpho/GMorpho.cu>
#undef private
#undef protected

using namespace MorphoGraphics;

namespace {

void set_err(char* err, int cap, const std::string& m) {
  if (err && cap > 0) {
    strncpy(err, m.c_str(), (size_t)cap - 1);
    err[cap - 1] = 0;
  }
}

template <typename T>
void free_dev(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

void free_grid(Grid& g) {
  GridGPU gg = g.grid_gpu();
  if (gg.voxels) cudaFree(gg.voxels);
  if (gg.tex_mipmap) cudaDestroyTextureObject(gg.tex_mipmap);
  if (gg.mipmapped_array) cudaFreeMipmappedArray(gg.mipmapped_array);
  gg.voxels = nullptr;
  gg.tex_mipmap = 0;
  gg.mipmapped_array = nullptr;
  g.set_grid_gpu(gg);
}

// The reference's destructors free nothing (Grid.cu:103-105,
// GMorpho.cu:97-99); release what one update allocated.
void release(GMorpho& g, ScaleField& sf) {
  free_grid(g.input_grid_);
  free_grid(g.dilation_grid_);
  free_grid(g.dilation_contour_grid_);
  free_grid(g.closing_grid_);
  free_dev(g.global_warp_counter_);
  free_dev(g.grid_2x2x2_uint_);
  free_dev(g.mcm_contour_indices_);
  free_dev(g.mcm_contour_values_);
  free_dev(g.mcm_contour_non_empty_);
  free_dev(g.mcm_compact_contour_values_);
  free_dev(g.mcm_compact_contour_indices_);
  free_dev(g.mcm_compact_contour_neigh_indices_);
  free_dev(g.mcm_compact_contour_neigh_morpho_centroids_);
  free_dev(g.mcm_vertices);
  free_dev(g.mcm_normals);
  free_dev(g.mcm_bilateral_normals);
  free_dev(g.mcm_triangles);
  free_dev(sf.scale_grid_);
}

}  // namespace

// X: res^3 packed bytes; scale: (2 res)^3 int8 radii; data_res: 3 ints.
// asymmetric: cube dilation (use_asymmetric_closing, 200 bilateral
// iterations) instead of the sphere (20 iterations).  D, S, C: res^3 bytes
// (dilation, its contour as TransformToContour leaves it, closing).  V, N:
// 3 floats per vertex, T: 3 uint32 per triangle, up to cap_v / cap_t; *nv,
// *nt get the counts.  Returns 0, or -1 with a message in err.
extern "C" int gmref_update(const uint8_t* X, const int8_t* scale, int res, const int* data_res, int asymmetric,
                            int bilateral, uint8_t* D, uint8_t* S, uint8_t* C, float* V, float* N, uint32_t* T,
                            int64_t cap_v, int64_t cap_t, int64_t* nv, int64_t* nt, char* err, int errcap) {
  GMorpho g;
  ScaleField sf;
  int rc = 0;
  try {
    const float cell = 1.f / (float)res;
    const Vec3f lo(0.f, 0.f, 0.f), hi(1.f, 1.f, 1.f);
    const Vec3ui rv(res, res, res), dr(data_res[0], data_res[1], data_res[2]);
    // what Load takes from the voxelizer (GMorpho.cu:7748-7752)
    g.input_grid_.Init(AxisAlignedBoundingBox(lo, hi), rv, dr, cell);
    if (cudaMemcpy(g.input_grid_.grid_gpu().voxels, X, (size_t)res * res * res, cudaMemcpyHostToDevice) !=
        cudaSuccess)
      throw std::runtime_error("input upload");
    g.bbox_ = g.input_grid_.bbox();
    g.res_ = g.input_grid_.res();
    g.data_res_ = g.input_grid_.data_res();
    g.cell_size_ = g.input_grid_.cell_size();
    // the rest of Load (GMorpho.cu:7757-7772)
    g.dilation_grid_.Init(g.bbox_, g.res_, g.data_res_, g.cell_size_);
    g.dilation_grid_.CopyVoxelsFrom(g.input_grid_);
    g.closing_grid_.Init(g.bbox_, g.res_, g.data_res_, g.cell_size_);
    g.closing_grid_.CopyVoxelsFrom(g.dilation_grid_);
    g.dilation_contour_grid_.Init(g.bbox_, g.res_, g.data_res_, g.cell_size_);
    g.ErodeAllocation();
    g.ExtractClosingMeshAllocation();
    g.set_use_asymmetric_closing(asymmetric != 0);
    g.set_use_frame_field(false);
    g.set_bilateral_filtering(bilateral != 0);

    // the scale field over the fine grid (BroxyViewer.cpp:131-137), its
    // radii replaced by the caller's; one brush point so that the pyramid
    // build's upload of the points (Grid.cu:1053-1056) has an element
    sf.Init(lo, hi, Vec3ui(2 * res, 2 * res, 2 * res), 0.5f * cell);
    sf.set_global_scale(cell);  // floor(2 gs / cell) = 2 > 1: the morphology runs (GMorpho.cu:7783)
    sf.AddPoint(Vec3f(0.5f, 0.5f, 0.5f), cell);
    if (cudaMemcpy(sf.scale_grid(), scale, (size_t)8 * res * res * res, cudaMemcpyHostToDevice) != cudaSuccess)
      throw std::runtime_error("scale upload");

    FrameField ff;  // not read: use_frame_field is off
    Mesh mesh;
    g.Update(mesh, sf, ff);
    if (cudaDeviceSynchronize() != cudaSuccess) throw std::runtime_error("device error after Update");

    const size_t cells = (size_t)res * res * res;
    if (D) cudaMemcpy(D, g.dilation_grid_.grid_gpu().voxels, cells, cudaMemcpyDeviceToHost);
    if (S) cudaMemcpy(S, g.dilation_contour_grid_.grid_gpu().voxels, cells, cudaMemcpyDeviceToHost);
    if (C) cudaMemcpy(C, g.closing_grid_.grid_gpu().voxels, cells, cudaMemcpyDeviceToHost);
    *nv = (int64_t)mesh.P().size();
    *nt = (int64_t)mesh.T().size();
    if (*nv <= cap_v && *nt <= cap_t) {
      for (int64_t i = 0; i < *nv; i++)
        for (int k = 0; k < 3; k++) {
          V[3 * i + k] = mesh.P()[i][k];
          N[3 * i + k] = mesh.N()[i][k];
        }
      for (int64_t i = 0; i < *nt; i++)
        for (int k = 0; k < 3; k++) T[3 * i + k] = mesh.T()[i][k];
    }
    if (cudaGetLastError() != cudaSuccess) throw std::runtime_error("CUDA error reading results");
  } catch (const GMorpho::Exception& e) {
    set_err(err, errcap, e.msg());
    rc = -1;
  } catch (const Grid::Exception& e) {
    set_err(err, errcap, e.msg());
    rc = -1;
  } catch (const std::exception& e) {
    set_err(err, errcap, e.what());
    rc = -1;
  }
  release(g, sf);
  return rc;
}
