// GMorpho.h — the reference's GMorpho class (GMorpho/GMorpho.h:48-170) over
// libgmorpho_gb300.  Same public methods; the closing runs the GB300
// kernels through the C ABI (gmorpho_gb300.h).
#pragma once
#include <string>

#include "BoundingVolume.h"
#include "FrameField.h"
#include "Grid.h"
#include "Mesh.h"
#include "ScaleField.h"
#include "Voxelizer.h"

struct gm_ctx;

namespace MorphoGraphics {

class GMorpho {
 public:
  class Exception {
   public:
    inline Exception(const std::string& msg) : msg_("GMorpho Error: " + msg) {}
    inline const std::string& msg() const { return msg_; }

   protected:
    std::string msg_;
  };

  typedef MorphoGraphics::AxisAlignedBoundingBox BoundingBox;

  GMorpho();
  virtual ~GMorpho();

  // the grid's box after Load (GMorpho.h:63)
  const BoundingBox& bbox() const { return bbox_; }
  const Vec3f& bbox_min() const { return input_grid_.bbox_min(); }
  const Vec3f& bbox_max() const { return input_grid_.bbox_max(); }
  const Vec3ui& res() const { return input_grid_.res(); }
  float cell_size() const { return input_grid_.cell_size(); }
  float se_size() const { return se_size_; }
  void set_se_size(float se_size) { se_size_ = se_size; }
  void set_use_asymmetric_closing(bool v) { use_asymmetric_closing_ = v; }
  bool use_asymmetric_closing() { return use_asymmetric_closing_; }
  void set_use_frame_field(bool v) { use_frame_field_ = v; }
  bool use_frame_field() { return use_frame_field_; }
  void set_bilateral_filtering(bool v) { bilateral_filtering_ = v; }
  Mesh get_morpho_mesh() { return morpho_mesh_; }
  // The reference exposes its internal 4V-byte splat map here (scratch of
  // its mesh extraction, GMorpho.cu:6787-6834, read by nothing outside
  // GMorpho); this library does not build one (it keeps one vertex offset
  // per cell instead), so there is no such buffer: nullptr.
  unsigned int* grid_2x2x2_uint() { return nullptr; }
  // GM_REF (default) reproduces the reference grids; GM_EXACT = 1 gives the
  // pure ball closing.
  void set_mode(int mode) { mode_ = mode; }

  void Load(const float* P, const float* N, int num_of_vertices, const unsigned int* T, int num_of_faces,
            int base_res, float se_size);
  void Update(Mesh& mesh, const ScaleField& scale_field, const FrameField& frame_field);
  void DilateBySphereMipmap(const ScaleField& scale_field);
  void DilateByCubeMipmap(const ScaleField& scale_field);
  // the rotated-cube dilation and the sphere erosion in one call (closing_grid())
  void DilateByRotCubeMipmap(const ScaleField& scale_field, const FrameField& frame_field);
  void ErodeBySphereMipmap(const ScaleField& scale_field);
  void ErodeAllocation() {}
  void ExtractClosingMeshAllocation() {}

  void Update(Mesh& mesh, float se_size);
  void DilateByCubeMipmap(float se_size);
  void DilateBySphereMipmap(float se_size);
  void ErodeBySphereMipmap(float se_size);
  void ExtractClosingMesh();
  void ExtractClosingMesh(Mesh& mesh, int num_bilateral_iters = 20);
  // erosion of the last dilation by a BVH over its contour, uniform radius
  // floor(2 se_size / cell_size) (GMorpho.cu:9308-9401), into closing_grid()
  void ErodeByBVH(float se_size);

  // device grids of the last update (packed 2x2x2 bytes)
  const Grid& input_grid() const { return input_grid_; }
  const Grid& dilation_grid() const { return dilation_grid_; }
  const Grid& closing_grid() const { return closing_grid_; }

 private:
  void close(const ScaleField* sf, int uniform_radius, int se);
  void close_rotcube(const ScaleField& sf, const FrameField& ff);
  void check(int status, const char* what);

  Voxelizer voxelizer_;
  BoundingBox bbox_;
  float se_size_ = 0.f;
  bool use_asymmetric_closing_ = false;
  bool use_frame_field_ = false;
  bool bilateral_filtering_ = true;
  int mode_ = 0;
  Mesh morpho_mesh_;
  Grid input_grid_, dilation_grid_, closing_grid_;
  gm_ctx* ctx_ = nullptr;
};

}  // namespace MorphoGraphics
