// Voxelizer.h — mesh to packed grid (reference GMorpho/Voxelizer.h).  The
// OpenGL shader path of the reference is replaced by CUDA kernels
// (gm_voxelize); VoxelizeConservative keeps its signature.
#pragma once
#include <vector>

#include "Grid.h"
#include "Mesh.h"

namespace MorphoGraphics {

class Voxelizer {
 public:
  Voxelizer() {}
  virtual ~Voxelizer();
  void Load(const float* P, const float* N, int num_of_vertices, const unsigned int* T, int num_of_faces);
  void VoxelizeConservative(int base_res, float margin);
  const Grid& grid() const { return grid_; }
  Grid& grid() { return grid_; }

 private:
  std::vector<float> P_;
  std::vector<unsigned int> T_;
  Grid grid_;
};

}  // namespace MorphoGraphics
