// MarchingCubesMesher.h — contour marching cubes (reference
// GMorpho/MarchingCubesMesher.h:647-764, global namespace).  createMesh3D
// meshes a packed closed grid at isovalue 0.95 in the reference's emission
// order; the mesh stays on the device (getDeviceMesh).
#pragma once
#include "gmorpho/Grid.h"

struct gm_ctx;

class MarchingCubesMesher {
 public:
  class Grid {
   public:
    Grid(const MorphoGraphics::Vec3f& origin, float cell_size_x, float cell_size_y, float cell_size_z,
         unsigned int nx, unsigned int ny, unsigned int nz)
        : origin_(origin), cs_{cell_size_x, cell_size_y, cell_size_z}, n_{nx, ny, nz} {}
    const MorphoGraphics::Vec3f& getOrigin() const { return origin_; }
    float getCellSizeX() const { return cs_[0]; }
    unsigned int getNbCellsX() const { return n_[0]; }
    unsigned int getNbCellsY() const { return n_[1]; }
    unsigned int getNbCellsZ() const { return n_[2]; }

   private:
    MorphoGraphics::Vec3f origin_;
    float cs_[3];
    unsigned int n_[3];
  };

  explicit MarchingCubesMesher(Grid* grid);
  ~MarchingCubesMesher();
  // d_voxels: packed grid of (nx/2)^3 bytes (fine grid nx^3)
  void createMesh3D(const unsigned char* d_voxels, int bilateral_iters = 0);
  void getDeviceMesh(const float** V, const float** N, unsigned int* VSize, const unsigned int** T,
                     unsigned int* TSize) const;

 private:
  Grid* grid_;
  gm_ctx* ctx_ = nullptr;
  const float* V_ = nullptr;
  const float* N_ = nullptr;
  const unsigned int* T_ = nullptr;
  unsigned int nv_ = 0, nt_ = 0;
};
