// Mesh.h — host mesh with the reference's P()/N()/T() accessors and OFF
// I/O (reference Common/Mesh.h:580-640).  Only what the GMorpho boundary
// uses: positions, normals, triangles.
#pragma once
#include <cstdio>
#include <ostream>
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
template <typename T>
inline Vec3<T> operator*(T s, const Vec3<T>& a) {
  return Vec3<T>(s * a[0], s * a[1], s * a[2]);
}
template <typename T>
inline Vec3<T> operator*(const Vec3<T>& a, T s) {
  return s * a;
}
template <typename T>
inline Vec3<T> operator+(const Vec3<T>& a, const Vec3<T>& b) {
  return Vec3<T>(a[0] + b[0], a[1] + b[1], a[2] + b[2]);
}
template <typename T>
inline Vec3<T> operator-(const Vec3<T>& a, const Vec3<T>& b) {
  return Vec3<T>(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
}
template <typename T>
inline std::ostream& operator<<(std::ostream& os, const Vec3<T>& a) {
  return os << a[0] << " " << a[1] << " " << a[2];
}
typedef Vec3<float> Vec3f;
typedef Vec3<unsigned int> Vec3ui;
typedef Vec3<int> Vec3i;

class Mesh {
 public:
  class Exception {
   public:
    inline Exception(const std::string& msg) : msg_("Mesh Error: " + msg) {}
    inline const std::string& msg() const { return msg_; }

   protected:
    std::string msg_;
  };

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
  // PN: float32 position + normal per vertex (reference Mesh::loadPN /
  // storePN, Common/Mesh.h:638-673)
  bool loadPN(const std::string& path);
  bool storePN(const std::string& path) const;
  // binary little-endian PLY with normals
  bool storePLY(const std::string& path) const;
  // by extension (".off", ".pn", ".ply" for store); throws Exception on
  // an unknown format or an I/O failure (reference Mesh::load / store)
  void load(const std::string& path);
  void store(const std::string& path) const;

 private:
  std::vector<Vec3f> P_, N_;
  std::vector<Vec3ui> T_;
};

}  // namespace MorphoGraphics
