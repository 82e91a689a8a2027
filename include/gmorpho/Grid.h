// Grid.h — packed 2x2x2 grid on the device (reference GMorpho/Grid.h:40-160).
// GridGPU keeps the reference fields that still have a meaning here:
// bbox, res, data_res, cell_size, the voxel bytes and the texel pyramid.
#pragma once
#include <stdint.h>

#include <string>

#include "Mesh.h"
#include "ScaleField.h"

struct GridGPU {
  float bbox_min[3];
  float bbox_max[3];
  unsigned int res[3];
  unsigned int data_res[3];
  float cell_size;
  unsigned char* voxels;      // res^3 packed bytes (device)
  unsigned long long* pyramid;  // texel pyramid levels 0..log2(res) (device), or NULL
  int max_mipmap_level;
};

namespace MorphoGraphics {

class Grid {
 public:
  class Exception {
   public:
    inline Exception(const std::string& msg) : msg_("Grid Error: " + msg) {}
    inline const std::string& msg() const { return msg_; }

   protected:
    std::string msg_;
  };

  Grid();
  virtual ~Grid();
  // device memory is owned: grids are not copied implicitly (use CopyVoxelsFrom)
  Grid(const Grid&) = delete;
  Grid& operator=(const Grid&) = delete;
  const Vec3f& bbox_min() const { return bbox_min_; }
  const Vec3f& bbox_max() const { return bbox_max_; }
  const Vec3ui& res() const { return res_; }
  const Vec3ui& data_res() const { return data_res_; }
  float cell_size() const { return cell_size_; }
  GridGPU grid_gpu() const;

  void Init(const Vec3f& bbox_min, const Vec3f& bbox_max, const Vec3ui& res, const Vec3ui& data_res,
            float cell_size);
  void SetGridValue(unsigned char value);
  void CopyVoxelsFrom(const Grid& grid);
  void BuildTexMipmaps(const ScaleField& scale_field);
  void BuildTexMipmaps(float se_size);
  // the 6-connected outer contour of the grid's voxels (in place)
  void TransformToContour();
  void Free();

 private:
  Vec3f bbox_min_, bbox_max_;
  Vec3ui res_, data_res_;
  float cell_size_ = 0.f;
  unsigned char* voxels_ = nullptr;
  unsigned long long* pyramid_ = nullptr;
};

}  // namespace MorphoGraphics
