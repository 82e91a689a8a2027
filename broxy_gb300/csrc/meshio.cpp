// meshio.cpp — host mesh files (reference Common/Mesh.h:580-673: OFF and
// PN stores) plus binary PLY, for meshes and served patches.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gmorpho_gb300.h"

namespace {

bool ends_with(const std::string& s, const char* suf) {
  const size_t n = std::strlen(suf);
  return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

void put_u32(std::vector<uint8_t>& b, uint32_t v) {
  for (int k = 0; k < 4; k++) b.push_back((uint8_t)(v >> (8 * k)));
}
void put_f32(std::vector<uint8_t>& b, float f) {
  uint32_t v;
  std::memcpy(&v, &f, 4);
  put_u32(b, v);
}

}  // namespace

extern "C" gm_status gm_mesh_store(const char* path, const float* V, const float* N, int64_t nv, const uint32_t* T,
                                   int64_t nt, int32_t drop_unused) {
  if (!path || nv < 0 || nt < 0 || (nv > 0 && !V) || (nt > 0 && !T) || nv > 0xffffffffLL) return GM_ERR_INVALID_ARGUMENT;
  const std::string p(path);
  const bool off = ends_with(p, ".off"), pn = ends_with(p, ".pn"), ply = ends_with(p, ".ply");
  if (!off && !pn && !ply) return GM_ERR_INVALID_ARGUMENT;
  if ((pn || ply) && nv > 0 && !N) return GM_ERR_INVALID_ARGUMENT;
  for (int64_t i = 0; i < 3 * nt; i++)
    if ((int64_t)T[i] >= nv) return GM_ERR_INVALID_ARGUMENT;
  // vertex renumbering (identity unless unused vertices are dropped)
  std::vector<uint32_t> remap;
  int64_t kept = nv;
  if (drop_unused) {
    remap.assign((size_t)nv, 0xffffffffu);
    for (int64_t i = 0; i < 3 * nt; i++) remap[T[i]] = 0;
    kept = 0;
    for (int64_t v = 0; v < nv; v++)
      if (remap[v] == 0) remap[v] = (uint32_t)kept++;
  }
  auto vid = [&](uint32_t v) { return drop_unused ? remap[v] : v; };
  auto used = [&](int64_t v) { return !drop_unused || remap[v] != 0xffffffffu; };
  FILE* f = std::fopen(path, off ? "w" : "wb");
  if (!f) return GM_ERR_INVALID_ARGUMENT;
  bool ok = true;
  if (off) {
    ok = std::fprintf(f, "OFF\n%lld %lld 0\n", (long long)kept, (long long)nt) > 0;
    for (int64_t v = 0; v < nv && ok; v++)
      if (used(v)) ok = std::fprintf(f, "%.9g %.9g %.9g\n", V[3 * v], V[3 * v + 1], V[3 * v + 2]) > 0;
    for (int64_t t = 0; t < nt && ok; t++)
      ok = std::fprintf(f, "3 %u %u %u\n", vid(T[3 * t]), vid(T[3 * t + 1]), vid(T[3 * t + 2])) > 0;
  } else {
    std::vector<uint8_t> buf;
    if (ply) {
      char head[512];
      std::snprintf(head, sizeof(head),
                    "ply\nformat binary_little_endian 1.0\nelement vertex %lld\nproperty float x\nproperty float y\n"
                    "property float z\nproperty float nx\nproperty float ny\nproperty float nz\nelement face %lld\n"
                    "property list uchar uint vertex_indices\nend_header\n",
                    (long long)kept, (long long)nt);
      buf.insert(buf.end(), head, head + std::strlen(head));
    }
    for (int64_t v = 0; v < nv; v++) {
      if (!used(v)) continue;
      for (int k = 0; k < 3; k++) put_f32(buf, V[3 * v + k]);
      for (int k = 0; k < 3; k++) put_f32(buf, N[3 * v + k]);
      if (buf.size() > (1u << 24)) {
        ok = ok && std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
        buf.clear();
      }
    }
    if (ply)
      for (int64_t t = 0; t < nt; t++) {
        buf.push_back(3);
        for (int k = 0; k < 3; k++) put_u32(buf, vid(T[3 * t + k]));
        if (buf.size() > (1u << 24)) {
          ok = ok && std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
          buf.clear();
        }
      }
    ok = ok && std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GM_OK : GM_ERR_INVALID_ARGUMENT;
}
