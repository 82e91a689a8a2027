// Stand-in for the reference's Common/Mesh.h in the reference build
// (oracle/refbuild/build_ref.py): the container part that GMorpho.cu uses
// (P, N, T vectors, clear, recomputeNormals); the drawing, VBO and file I/O
// members of the original are not needed by the morphology path.
#pragma once
#include <cmath>
#include <string>
#include <vector>

#include <Common/Vec3.h>

namespace MorphoGraphics {

class Mesh {
 public:
  class Exception {
   public:
    inline Exception(const std::string& msg) : msg_("MorphoGraphics Mesh Exception: " + msg) {}
    inline const std::string& msg() const { return msg_; }

   private:
    std::string msg_;
  };
  typedef Vec3<unsigned int> Triangle;

  Mesh() {}
  virtual ~Mesh() {}
  std::vector<Vec3f>& P() { return P_; }
  std::vector<Vec3f>& N() { return N_; }
  std::vector<Triangle>& T() { return T_; }
  const std::vector<Vec3f>& P() const { return P_; }
  const std::vector<Vec3f>& N() const { return N_; }
  const std::vector<Triangle>& T() const { return T_; }
  void clear() {
    P_.clear();
    N_.clear();
    T_.clear();
  }
  // area-weighted vertex normals from the triangles
  void recomputeNormals() {
    N_.assign(P_.size(), Vec3f(0.f, 0.f, 0.f));
    for (const Triangle& t : T_) {
      Vec3f a = P_[t[1]] - P_[t[0]], b = P_[t[2]] - P_[t[0]];
      Vec3f n(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
      for (int k = 0; k < 3; k++) N_[t[k]] += n;
    }
    for (Vec3f& n : N_) {
      float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      if (l > 0.f) n /= l;
    }
  }

 private:
  std::vector<Vec3f> P_, N_;
  std::vector<Triangle> T_;
};

}  // namespace MorphoGraphics
