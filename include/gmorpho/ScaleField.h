// ScaleField.h — per-fine-voxel radius grid (reference GMorpho/ScaleField.h).
// scale_grid() is a device char grid of res^3 fine voxels, as in the
// reference; UpdateGrid applies the last brush point, UpdateGridGlobalScale
// fills floor(global_scale / cell_size).
#pragma once
#include <string>
#include <vector>

#include "Mesh.h"

namespace MorphoGraphics {

typedef enum { NO_EDITION, MAX_BRUSH, MIN_BRUSH, ZERO_BRUSH } EditMode;

class ScaleField {
 public:
  class Exception {
   public:
    inline Exception(const std::string& msg) : msg_("ScaleField Error: " + msg) {}
    inline const std::string& msg() const { return msg_; }

   protected:
    std::string msg_;
  };

  class ScalePoint {
   public:
    ScalePoint() {}
    ScalePoint(const Vec3f& position, float scale) : position_(position), scale_(scale), support_(scale) {}
    ScalePoint(const Vec3f& position, float scale, float support)
        : position_(position), scale_(scale), support_(support) {}
    const Vec3f& position() const { return position_; }
    float scale() const { return scale_; }
    float support() const { return support_; }
    EditMode edit_mode() const { return edit_mode_; }
    void set_position(const Vec3f& p) { position_ = p; }
    void set_scale(float s) { scale_ = s; }
    void set_support(float s) { support_ = s; }
    void set_edit_mode(EditMode m) { edit_mode_ = m; }

   private:
    Vec3f position_;
    float scale_ = 0.f, support_ = 0.f;
    EditMode edit_mode_ = MAX_BRUSH;
  };

  ScaleField() {}
  virtual ~ScaleField();

  float cell_size() const { return cell_size_; }
  const Vec3f& bbox_min() const { return bbox_min_; }
  const Vec3f& bbox_max() const { return bbox_max_; }
  const Vec3ui& res() const { return res_; }
  float global_scale() const { return global_scale_; }
  void set_global_scale(float s) { global_scale_ = s; }
  void AddPoint(const Vec3f& position, float scale) { points_.push_back(ScalePoint(position, scale)); }
  void AddPoint(const Vec3f& position, float scale, float support) {
    points_.push_back(ScalePoint(position, scale, support));
  }
  const std::vector<ScalePoint>& points() const { return points_; }
  std::vector<ScalePoint>& points() { return points_; }
  int GetNumberOfPoints() const { return (int)points_.size(); }
  char* scale_grid() const { return scale_grid_; }

  void GetScaleGridCPU(char** scale_grid_cpu_ptr);
  void Init(const Vec3f& bbox_min, const Vec3f& bbox_max, const Vec3ui& res, float cell_size);
  void UpdateGrid();
  void UpdateGridGlobalScale();

 private:
  std::vector<ScalePoint> points_;
  float global_scale_ = 0.f;
  Vec3f bbox_min_, bbox_max_;
  Vec3ui res_;
  float cell_size_ = 0.f;
  char* scale_grid_ = nullptr;
};

}  // namespace MorphoGraphics
