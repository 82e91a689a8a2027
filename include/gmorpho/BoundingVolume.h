// BoundingVolume.h — the axis-aligned box that GMorpho::bbox() returns
// (reference Common/BoundingVolume.h:104-160, the accessors its callers
// use: min(), max(), center(), extents).
#pragma once
#include <algorithm>

#include "Mesh.h"

namespace MorphoGraphics {

class AxisAlignedBoundingBox {
 public:
  AxisAlignedBoundingBox() {}
  explicit AxisAlignedBoundingBox(const Vec3f& p) : min_(p), max_(p) {}
  AxisAlignedBoundingBox(const Vec3f& lo, const Vec3f& hi) : min_(lo), max_(hi) {}
  virtual ~AxisAlignedBoundingBox() {}
  const Vec3f& min() const { return min_; }
  const Vec3f& max() const { return max_; }
  Vec3f center() const { return Vec3f(0.5f * (min_[0] + max_[0]), 0.5f * (min_[1] + max_[1]), 0.5f * (min_[2] + max_[2])); }
  float width() const { return max_[0] - min_[0]; }
  float height() const { return max_[1] - min_[1]; }
  float length() const { return max_[2] - min_[2]; }
  float size() const { return std::max(width(), std::max(height(), length())); }
  bool contains(const Vec3f& p) const {
    for (int i = 0; i < 3; i++)
      if (!(p[i] >= min_[i] && p[i] <= max_[i])) return false;
    return true;
  }

 private:
  Vec3f min_, max_;
};

}  // namespace MorphoGraphics
