// The reference viewer's calls into GMorpho, in the forms it writes them
// (BroxyViewer.cpp:121-157 mesh load and scale/frame field set-up,
// :180-193 closing toggles, :197-233 base scale steps), compiled against
// include/gmorpho/.  Prints the numbers the Python test checks.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <vector>

#include "gmorpho/GMorpho.h"

using namespace MorphoGraphics;

static const int kVoxelRes = 64;     // the viewer's VOXEL_RESOLUTION, smaller
static const float kMaxSe = 0.3f;    // MAX_SE_SIZE
static const float kInitSe = 0.05f;  // INITIAL_SE_SIZE

static GMorpho gmorpho;
static FrameField frame_field;

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  Mesh mesh, morpho;
  if (!mesh.loadOFF(argv[1])) return 2;
  mesh.N().assign(mesh.P().size(), Vec3f(0.f, 0.f, 1.f));
  ScaleField scale_field;
  try {
    const std::vector<Vec3f>& positions = mesh.P();
    const std::vector<Vec3f>& normals = mesh.N();
    const std::vector<Vec3<unsigned int> >& triangles = mesh.T();
    gmorpho.set_bilateral_filtering(true);
    gmorpho.Load(&positions[0][0], &normals[0][0], positions.size(), &triangles[0][0], triangles.size(), kVoxelRes,
                 kMaxSe);
    Vec3f bbox_min = gmorpho.bbox().min();
    Vec3f bbox_max = gmorpho.bbox().max();
    Vec3ui res = ((unsigned int)2) * gmorpho.res();
    float cell_size = 0.5f * gmorpho.cell_size();
    scale_field.set_global_scale(kInitSe);
    scale_field.Init(bbox_min, bbox_max, res, cell_size);
    scale_field.UpdateGridGlobalScale();
    gmorpho.set_use_asymmetric_closing(true);
    gmorpho.set_use_frame_field(false);
    Vec3i frame_field_res(gmorpho.res()[0] / 16, gmorpho.res()[1] / 16, gmorpho.res()[2] / 16);
    std::cout << "frame_field_res : " << frame_field_res << std::endl;
    frame_field.Init(bbox_min, bbox_max, frame_field_res, FrameField::BiHarmonicSystem);
    frame_field.Generate(false, false);
    gmorpho.Update(morpho, scale_field, frame_field);
    const size_t t_asym = morpho.T().size();

    // toggles
    gmorpho.set_use_asymmetric_closing(false);
    gmorpho.Update(morpho, scale_field, frame_field);
    const size_t t_sym = morpho.T().size();
    gmorpho.set_use_frame_field(true);
    gmorpho.Update(morpho, scale_field, frame_field);

    // one base scale step up, then down
    float global_scale = scale_field.global_scale();
    global_scale += 0.5f * gmorpho.cell_size();
    global_scale = std::max(global_scale, 0.5f * gmorpho.cell_size());
    global_scale = std::min(global_scale, kMaxSe);
    if ((global_scale != kMaxSe) && (global_scale != 0.5f * gmorpho.cell_size())) {
      scale_field.set_global_scale(global_scale);
      scale_field.UpdateGridGlobalScale();
      gmorpho.Update(morpho, scale_field, frame_field);
    }
    const size_t t_up = morpho.T().size();
    global_scale = scale_field.global_scale();
    global_scale -= 0.5f * gmorpho.cell_size();
    global_scale = std::max(global_scale, 0.5f * gmorpho.cell_size());
    global_scale = std::min(global_scale, kMaxSe);
    if ((global_scale != kMaxSe) && (global_scale != 0.5f * gmorpho.cell_size())) {
      scale_field.set_global_scale(global_scale);
      scale_field.UpdateGridGlobalScale();
      gmorpho.Update(morpho, scale_field, frame_field);
    }
    const size_t t_down = morpho.T().size();

    // the box is the grid's
    for (int i = 0; i < 3; i++)
      if (bbox_min[i] != gmorpho.bbox_min()[i] || bbox_max[i] != gmorpho.bbox_max()[i]) return 4;

    // BVH erosion of the last uniform-radius dilation (GMorpho::ErodeByBVH)
    gmorpho.DilateBySphereMipmap(kInitSe);
    gmorpho.ErodeByBVH(kInitSe);
    const size_t cells = (size_t)gmorpho.res()[0] * gmorpho.res()[1] * gmorpho.res()[2];
    if (argc > 2) {
      std::vector<unsigned char> h(cells);
      auto dump = [&](const char* name, const Grid& g) {
        if (cudaMemcpy(h.data(), g.grid_gpu().voxels, cells, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
        FILE* f = fopen((std::string(argv[2]) + "/" + name).c_str(), "wb");
        if (!f) return false;
        fwrite(h.data(), 1, cells, f);
        fclose(f);
        return true;
      };
      if (!dump("input.bin", gmorpho.input_grid()) || !dump("dilation.bin", gmorpho.dilation_grid()) ||
          !dump("bvh_closing.bin", gmorpho.closing_grid()))
        return 5;
    }
    const Vec3ui& dr = gmorpho.input_grid().data_res();
    printf("%zu %zu %zu %zu %u %d %d %u %u %u\n", t_asym, t_sym, t_up, t_down, gmorpho.res()[0],
           (int)std::floor(2.f * kInitSe / gmorpho.cell_size()), gmorpho.grid_2x2x2_uint() == nullptr, dr[0], dr[1],
           dr[2]);
  } catch (const GMorpho::Exception& e) {
    fprintf(stderr, "%s\n", e.msg().c_str());
    return 1;
  } catch (const FrameField::Exception& e) {
    fprintf(stderr, "%s\n", e.msg().c_str());
    return 1;
  } catch (const Grid::Exception& e) {
    fprintf(stderr, "%s\n", e.msg().c_str());
    return 1;
  }
  return 0;
}
