// FrameField.h — the reference's frame field (GMorpho/FrameField.h) with
// the BiHarmonicSystem method, over libgmorpho_gb300 (gm_frame_field_*): a
// quaternion per node of a res^3 lattice over the box, interpolating up to
// 20 hard-constrained rotations.  quats_pong() is the device field that
// GMorpho's rotated-cube dilation reads.  The OpenGL drawing helpers and
// the LocalOptimization method are not part of this library (Init with
// LocalOptimization throws "unsupported").
#pragma once
#include <string>
#include <vector>

#include "Mesh.h"

struct gm_frame_field;

namespace MorphoGraphics {

class FrameField {
 public:
  class Exception {
   public:
    inline Exception(const std::string& msg) : msg_("FrameField Error: " + msg) {}
    inline const std::string& msg() const { return msg_; }

   protected:
    std::string msg_;
  };

  class FramePoint {
   public:
    FramePoint() {}
    FramePoint(const Vec3f& position, const Vec3f& twist) : position_(position), twist_(twist) {}
    const Vec3f& position() const { return position_; }
    const Vec3f& twist() const { return twist_; }
    void set_position(const Vec3f& p) { position_ = p; }
    void set_twist(const Vec3f& t) { twist_ = t; }

   private:
    Vec3f position_, twist_;
  };

  typedef enum { BiHarmonicSystem, LocalOptimization } OptimMethod;

  FrameField() {}
  ~FrameField();
  FrameField(const FrameField&) = delete;
  FrameField& operator=(const FrameField&) = delete;

  float cell_size() const { return cell_size_; }
  const Vec3f& bbox_min() const { return bbox_min_; }
  const Vec3f& bbox_max() const { return bbox_max_; }
  const Vec3i& res() const { return res_; }

  void Init(const Vec3f& bbox_min, const Vec3f& bbox_max, const Vec3i& res, OptimMethod optim_method);
  void AddHardConstrainedPoint(const Vec3f& position, const Vec3f& e_x, const Vec3f& e_y, const Vec3f& e_z);
  void AddHardConstrainedPoint(const Vec3f& position, const Vec3f& twist);
  void UpdateHardConstrainedPoint(int i, const Vec3f& e_x, const Vec3f& e_y, const Vec3f& e_z);
  void UpdateHardConstrainedPoint(int i, const Vec3f& twist);
  Vec3f GetHardConstrainedPointTwist(int i);
  int GetHardConstrainedPointId(const Vec3f& position);
  int GetHardConstrainedPointId(const Vec3f& position, float eps_tolerance);
  const std::vector<FramePoint>& hc_points() const { return hc_points_; }
  int GetNumberOfHardConstrainedPoints() const { return (int)hc_points_.size(); }
  // device quaternions (x, y, z, w) per node, x-fastest; after Generate
  const float* quats_pong() const;
  void Generate(bool update_only, bool use_group_symmetry);
  static Vec3f RotationToTwistCayley(const Vec3f& e_x, const Vec3f& e_y, const Vec3f& e_z);

 private:
  gm_frame_field* ff_ = nullptr;
  Vec3f bbox_min_, bbox_max_;
  Vec3i res_;
  float cell_size_ = 0.f;
  std::vector<FramePoint> hc_points_;  // lattice positions, as the reference keeps them
};

}  // namespace MorphoGraphics
