// Mesh.h — host mesh with the reference's P()/N()/T() accessors and OFF
// I/O (reference Common/Mesh.h:580-640).  Only what the GMorpho boundary
// uses: positions, normals, triangles.
#pragma once
#include <cstdio>
#include <string>
#include <vector>

namespace MorphoGraphics {

template <typename T>
struct Vec3 {
  T v[3];
  Vec3() : v{T(0), T(0), T(0)} {}
  Vec3(T a, T b, T c) : v{a, b, c} {}
  T& operator[](int i) { return v[i]; }
  const T& operator[](int i) const { return v[i]; }
};
typedef Vec3<float> Vec3f;
typedef Vec3<unsigned int> Vec3ui;

class Mesh {
 public:
  std::vector<Vec3f>& P() { return P_; }
  const std::vector<Vec3f>& P() const { return P_; }
  std::vector<Vec3f>& N() { return N_; }
  const std::vector<Vec3f>& N() const { return N_; }
  std::vector<Vec3ui>& T() { return T_; }
  const std::vector<Vec3ui>& T() const { return T_; }
  void clear() { P_.clear(); N_.clear(); T_.clear(); }

  // OFF file I/O (reference Mesh::loadOFF / storeOFF)
  bool loadOFF(const std::string& path);
  bool storeOFF(const std::string& path) const;

 private:
  std::vector<Vec3f> P_, N_;
  std::vector<Vec3ui> T_;
};

}  // namespace MorphoGraphics
