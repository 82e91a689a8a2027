// gmorpho_classes.cpp — the reference's C++ classes (namespace
// MorphoGraphics: GMorpho, Grid, ScaleField, Voxelizer, Mesh; global
// MarchingCubesMesher) implemented over the C ABI of libgmorpho_gb300.
//
// Error behaviour follows the reference: failures throw the class's
// Exception (GMorpho/GMorpho.cu:50-56) carrying the library message.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>

#include "../../include/gmorpho/GMorpho.h"
#include "../../include/gmorpho/MarchingCubesMesher.h"
#include "../../include/gmorpho_gb300.h"

namespace {

// One context per device for the classes that have none of their own.
gm_ctx* shared_ctx() {
  static std::mutex mu;
  static gm_ctx* ctxs[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  if (dev < 0 || dev >= 64) return nullptr;
  if (!ctxs[dev] && gm_ctx_create(dev, &ctxs[dev]) != GM_OK) ctxs[dev] = nullptr;
  return ctxs[dev];
}

std::string message(gm_ctx* ctx, int status, const char* what) {
  std::string m = std::string(what) + ": " + gm_status_string((gm_status)status);
  if (ctx && gm_ctx_last_error(ctx)[0]) m += std::string(" (") + gm_ctx_last_error(ctx) + ")";
  return m;
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw MorphoGraphics::Grid::Exception(std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

namespace MorphoGraphics {

// ------------------------------------------------------------------ Mesh

bool Mesh::loadOFF(const std::string& path) {
  std::ifstream in(path);
  if (!in) return false;
  std::string head;
  in >> head;
  if (head != "OFF") return false;
  size_t nv = 0, nf = 0, ne = 0;
  in >> nv >> nf >> ne;
  P_.resize(nv);
  for (size_t i = 0; i < nv; i++) in >> P_[i][0] >> P_[i][1] >> P_[i][2];
  T_.clear();
  for (size_t i = 0; i < nf; i++) {
    unsigned int n, a, b, c;
    in >> n >> a >> b >> c;
    T_.push_back(Vec3ui(a, b, c));
    for (unsigned int k = 3; k < n; k++) {  // fan-triangulate polygons
      unsigned int d;
      in >> d;
      T_.push_back(Vec3ui(a, c, d));
      c = d;
    }
  }
  N_.clear();
  return (bool)in || in.eof();
}

bool Mesh::storeOFF(const std::string& path) const {
  std::ofstream out(path);
  if (!out) return false;
  out << "OFF\n" << P_.size() << " " << T_.size() << " 0\n";
  for (const Vec3f& p : P_) out << p[0] << " " << p[1] << " " << p[2] << "\n";
  for (const Vec3ui& t : T_) out << "3 " << t[0] << " " << t[1] << " " << t[2] << "\n";
  return (bool)out;
}

bool Mesh::loadPN(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::vector<float> buf;
  float tmp[6];
  while (std::fread(tmp, sizeof(float), 6, f) == 6) buf.insert(buf.end(), tmp, tmp + 6);
  std::fclose(f);
  const size_t n = buf.size() / 6;
  P_.resize(n);
  N_.resize(n);
  T_.clear();
  for (size_t i = 0; i < n; i++) {
    P_[i] = Vec3f(buf[6 * i], buf[6 * i + 1], buf[6 * i + 2]);
    N_[i] = Vec3f(buf[6 * i + 3], buf[6 * i + 4], buf[6 * i + 5]);
  }
  return true;
}

static bool store_via_abi(const Mesh& m, const std::string& path) {
  std::vector<float> n;
  const float* np = nullptr;
  if (m.N().size() == m.P().size()) {
    np = m.P().empty() ? nullptr : &m.N()[0][0];
  } else {
    n.assign(3 * m.P().size(), 0.f);  // no normals: zeros
    np = n.empty() ? nullptr : n.data();
  }
  return gm_mesh_store(path.c_str(), m.P().empty() ? nullptr : &m.P()[0][0], np, (int64_t)m.P().size(),
                       m.T().empty() ? nullptr : &m.T()[0][0], (int64_t)m.T().size(), 0) == GM_OK;
}

bool Mesh::storePN(const std::string& path) const { return store_via_abi(*this, path); }
bool Mesh::storePLY(const std::string& path) const { return store_via_abi(*this, path); }

static std::string extension(const std::string& path) {
  const size_t dot = path.find_last_of('.');
  return dot == std::string::npos ? std::string() : path.substr(dot);
}

void Mesh::load(const std::string& path) {
  const std::string ext = extension(path);
  bool ok;
  if (ext == ".off") ok = loadOFF(path);
  else if (ext == ".pn") ok = loadPN(path);
  else throw Exception("Error loading mesh: unrecognized file format.");
  if (!ok) throw Exception("Error loading mesh file: " + path);
}

void Mesh::store(const std::string& path) const {
  const std::string ext = extension(path);
  bool ok;
  if (ext == ".off") ok = storeOFF(path);
  else if (ext == ".pn") ok = storePN(path);
  else if (ext == ".ply") ok = storePLY(path);
  else throw Exception("Error storing mesh: unrecognized file format.");
  if (!ok) throw Exception("Error storing mesh file: " + path);
}

// ------------------------------------------------------------------ Grid

Grid::Grid() {}
Grid::~Grid() { Free(); }

void Grid::Free() {
  if (voxels_) cudaFree(voxels_);
  if (pyramid_) cudaFree(pyramid_);
  voxels_ = nullptr;
  pyramid_ = nullptr;
}

void Grid::Init(const Vec3f& bmin, const Vec3f& bmax, const Vec3ui& res, const Vec3ui& data_res, float cell_size) {
  if (res[0] != res[1] || res[0] != res[2]) throw Exception("grids are cubic");
  const size_t n = (size_t)res[0] * res[1] * res[2];
  if (voxels_ && res[0] == res_[0]) {
    // keep the allocation
  } else {
    Free();
    cuda_check(cudaMalloc(&voxels_, n), "Grid::Init");
  }
  bbox_min_ = bmin;
  bbox_max_ = bmax;
  res_ = res;
  data_res_ = data_res;
  cell_size_ = cell_size;
}

GridGPU Grid::grid_gpu() const {
  GridGPU g;
  for (int a = 0; a < 3; a++) {
    g.bbox_min[a] = bbox_min_[a];
    g.bbox_max[a] = bbox_max_[a];
    g.res[a] = res_[a];
    g.data_res[a] = data_res_[a];
  }
  g.cell_size = cell_size_;
  g.voxels = voxels_;
  g.pyramid = pyramid_;
  int l = 0;
  while ((1u << l) < res_[0]) l++;
  g.max_mipmap_level = l + 1;
  return g;
}

void Grid::SetGridValue(unsigned char value) {
  cuda_check(cudaMemset(voxels_, value, (size_t)res_[0] * res_[1] * res_[2]), "Grid::SetGridValue");
}

void Grid::CopyVoxelsFrom(const Grid& grid) {
  const size_t n = (size_t)res_[0] * res_[1] * res_[2];
  const size_t m = (size_t)grid.res_[0] * grid.res_[1] * grid.res_[2];
  if (n != m) throw Exception("impossible copy : size don't match");
  cuda_check(cudaMemcpy(voxels_, grid.voxels_, n, cudaMemcpyDeviceToDevice), "Grid::CopyVoxelsFrom");
}

static gm_grid_desc desc_of(const Grid& g) {
  gm_grid_desc d;
  for (int a = 0; a < 3; a++) {
    d.bbox_min[a] = g.bbox_min()[a];
    d.bbox_max[a] = g.bbox_max()[a];
    d.data_res[a] = (int32_t)g.data_res()[a];
  }
  d.res = (int32_t)g.res()[0];
  d.cell_size = g.cell_size();
  return d;
}

void Grid::BuildTexMipmaps(const ScaleField& sf) {
  gm_ctx* ctx = shared_ctx();
  if (!pyramid_) cuda_check(cudaMalloc(&pyramid_, 8 * (size_t)gm_pyramid_texels((int32_t)res_[0])), "pyramid");
  gm_grid_desc d = desc_of(*this);
  const int s = gm_pyramid_build(ctx, &d, voxels_, reinterpret_cast<const int8_t*>(sf.scale_grid()),
                                 (int32_t)std::floor(sf.global_scale() / sf.cell_size()),
                                 reinterpret_cast<uint64_t*>(pyramid_), nullptr);
  if (s != GM_OK) throw Exception(message(ctx, s, "Grid::BuildTexMipmaps"));
}

void Grid::BuildTexMipmaps(float se_size) {
  gm_ctx* ctx = shared_ctx();
  if (!pyramid_) cuda_check(cudaMalloc(&pyramid_, 8 * (size_t)gm_pyramid_texels((int32_t)res_[0])), "pyramid");
  gm_grid_desc d = desc_of(*this);
  const int s = gm_pyramid_build(ctx, &d, voxels_, nullptr, (int32_t)std::floor(2.f * se_size / cell_size_),
                                 reinterpret_cast<uint64_t*>(pyramid_), nullptr);
  if (s != GM_OK) throw Exception(message(ctx, s, "Grid::BuildTexMipmaps"));
}

void Grid::TransformToContour() {
  gm_ctx* ctx = shared_ctx();
  gm_grid_desc d = desc_of(*this);
  const int s = gm_contour(ctx, &d, voxels_, voxels_, GM_REF, nullptr);
  if (s != GM_OK) throw Exception(message(ctx, s, "Grid::TransformToContour"));
}

// ------------------------------------------------------------------ ScaleField

ScaleField::~ScaleField() {
  if (scale_grid_) cudaFree(scale_grid_);
}

void ScaleField::Init(const Vec3f& bbox_min, const Vec3f& bbox_max, const Vec3ui& res, float cell_size) {
  bbox_min_ = bbox_min;
  bbox_max_ = bbox_max;
  res_ = res;
  cell_size_ = cell_size;
  const size_t n = (size_t)res[0] * res[1] * res[2];
  if (!scale_grid_) cuda_check(cudaMalloc(&scale_grid_, n), "ScaleField::Init");
  cuda_check(cudaMemset(scale_grid_, 0, n), "ScaleField::Init");
}

void ScaleField::GetScaleGridCPU(char** out) {
  const size_t n = (size_t)res_[0] * res_[1] * res_[2];
  *out = new char[n];
  cuda_check(cudaMemcpy(*out, scale_grid_, n, cudaMemcpyDeviceToHost), "ScaleField::GetScaleGridCPU");
}

void ScaleField::UpdateGridGlobalScale() {
  gm_ctx* ctx = shared_ctx();
  const size_t n = (size_t)res_[0] * res_[1] * res_[2];
  const int s = gm_scalefield_fill(ctx, reinterpret_cast<int8_t*>(scale_grid_), (int64_t)n,
                                   (int32_t)std::floor(global_scale_ / cell_size_), nullptr);
  if (s != GM_OK) throw Exception(message(ctx, s, "ScaleField::UpdateGridGlobalScale"));
}

void ScaleField::UpdateGrid() {
  if (points_.empty()) return;
  gm_ctx* ctx = shared_ctx();
  const ScalePoint& p = points_.back();  // the reference applies the last point only
  const float bmin[3] = {bbox_min_[0], bbox_min_[1], bbox_min_[2]};
  const float pos[3] = {p.position()[0], p.position()[1], p.position()[2]};
  const gm_brush_mode mode = p.edit_mode() == MIN_BRUSH ? GM_BRUSH_MIN
                             : p.edit_mode() == ZERO_BRUSH ? GM_BRUSH_ZERO
                                                           : GM_BRUSH_MAX;
  if (p.edit_mode() == NO_EDITION) return;
  const int s = gm_scalefield_brush(ctx, reinterpret_cast<int8_t*>(scale_grid_), (int32_t)res_[0], bmin, cell_size_,
                                    pos, p.scale(), p.support(), global_scale_, mode, nullptr);
  if (s != GM_OK) throw Exception(message(ctx, s, "ScaleField::UpdateGrid"));
}

// ------------------------------------------------------------------ FrameField

FrameField::~FrameField() {
  if (ff_) gm_frame_field_destroy(ff_);
}

void FrameField::Init(const Vec3f& bbox_min, const Vec3f& bbox_max, const Vec3i& res, OptimMethod optim_method) {
  if (optim_method != BiHarmonicSystem) throw Exception("unsupported: LocalOptimization");
  gm_ctx* ctx = shared_ctx();
  if (ff_) gm_frame_field_destroy(ff_);
  ff_ = nullptr;
  hc_points_.clear();
  const float lo[3] = {bbox_min[0], bbox_min[1], bbox_min[2]}, hi[3] = {bbox_max[0], bbox_max[1], bbox_max[2]};
  const int s = gm_frame_field_create(ctx, lo, hi, res[0], &ff_);
  if (s != GM_OK) throw Exception(message(ctx, s, "FrameField::Init"));
  bbox_min_ = bbox_min;
  bbox_max_ = bbox_max;
  res_ = res;
  cell_size_ = std::max(std::fabs(bbox_max[0] - bbox_min[0]),
                        std::max(std::fabs(bbox_max[1] - bbox_min[1]), std::fabs(bbox_max[2] - bbox_min[2]))) /
               res[0];
}

Vec3f FrameField::RotationToTwistCayley(const Vec3f& e_x, const Vec3f& e_y, const Vec3f& e_z) {
  float t[3];
  const int s = gm_rotation_to_twist(&e_x[0], &e_y[0], &e_z[0], t);
  if (s != GM_OK) throw Exception("RotationToTwistCayley: half turn (R + I singular)");
  return Vec3f(t[0], t[1], t[2]);
}

void FrameField::AddHardConstrainedPoint(const Vec3f& position, const Vec3f& e_x, const Vec3f& e_y,
                                         const Vec3f& e_z) {
  AddHardConstrainedPoint(position, RotationToTwistCayley(e_x, e_y, e_z));
}

void FrameField::AddHardConstrainedPoint(const Vec3f& position, const Vec3f& twist) {
  if (!ff_) throw Exception("Init must come first");
  const int s = gm_frame_field_add_point(ff_, &position[0], &twist[0]);
  if (s == GM_ERR_CAPACITY) return;  // past 20 points the reference ignores the call
  if (s != GM_OK) throw Exception(message(shared_ctx(), s, "FrameField::AddHardConstrainedPoint"));
  float g[3], t[3];
  gm_frame_field_get_point(ff_, (int32_t)hc_points_.size(), g, t);
  hc_points_.push_back(FramePoint(Vec3f(g[0], g[1], g[2]), Vec3f(t[0], t[1], t[2])));
}

void FrameField::UpdateHardConstrainedPoint(int i, const Vec3f& e_x, const Vec3f& e_y, const Vec3f& e_z) {
  UpdateHardConstrainedPoint(i, RotationToTwistCayley(e_x, e_y, e_z));
}

void FrameField::UpdateHardConstrainedPoint(int i, const Vec3f& twist) {
  if (!ff_ || i < 0 || i >= (int)hc_points_.size()) return;
  gm_frame_field_update_point(ff_, i, &twist[0]);
  hc_points_[i].set_twist(twist);
}

Vec3f FrameField::GetHardConstrainedPointTwist(int i) {
  if (i >= 0 && i < (int)hc_points_.size()) return hc_points_[i].twist();
  return Vec3f(0, 0, 0);
}

int FrameField::GetHardConstrainedPointId(const Vec3f& position) {
  return GetHardConstrainedPointId(position, cell_size_);
}

// nearest hard-constrained node within eps_tolerance (FrameField.cu:103-126)
int FrameField::GetHardConstrainedPointId(const Vec3f& position, float eps_tolerance) {
  int best = -1;
  float best_d = std::numeric_limits<float>::max();
  for (int i = 0; i < (int)hc_points_.size(); i++) {
    float d2 = 0.f;
    for (int k = 0; k < 3; k++) {
      const float c = cell_size_ * hc_points_[i].position()[k] + bbox_min_[k];
      d2 += (position[k] - c) * (position[k] - c);
    }
    const float d = std::sqrt(d2);
    if (d < eps_tolerance && d < best_d) {
      best_d = d;
      best = i;
    }
  }
  return best;
}

const float* FrameField::quats_pong() const {
  if (!ff_) throw Exception("Init must come first");
  const float* q = nullptr;
  const int s = gm_frame_field_quats(ff_, &q, nullptr);
  if (s != GM_OK) throw Exception(message(shared_ctx(), s, "FrameField::quats_pong"));
  return q;
}

void FrameField::Generate(bool, bool) {
  if (!ff_) throw Exception("Init must come first");
  const int s = gm_frame_field_generate(ff_, nullptr, nullptr);
  if (s != GM_OK) throw Exception(message(shared_ctx(), s, "FrameField::Generate"));
}

// ------------------------------------------------------------------ Voxelizer

Voxelizer::~Voxelizer() {}

void Voxelizer::Load(const float* P, const float* N, int nv, const unsigned int* T, int nf) {
  (void)N;
  P_.assign(P, P + 3 * (size_t)nv);
  T_.assign(T, T + 3 * (size_t)nf);
}

void Voxelizer::VoxelizeConservative(int base_res, float margin) {
  gm_grid_desc d;
  int s = gm_grid_attributes(P_.data(), (int64_t)(P_.size() / 3), base_res, margin, &d);
  if (s != GM_OK) throw Grid::Exception("Voxelizer: bad mesh or resolution");
  grid_.Init(Vec3f(d.bbox_min[0], d.bbox_min[1], d.bbox_min[2]), Vec3f(d.bbox_max[0], d.bbox_max[1], d.bbox_max[2]),
             Vec3ui(d.res, d.res, d.res), Vec3ui(d.data_res[0], d.data_res[1], d.data_res[2]), d.cell_size);
  grid_.SetGridValue(0);
  float* dP = nullptr;
  unsigned int* dT = nullptr;
  cuda_check(cudaMalloc(&dP, sizeof(float) * P_.size()), "Voxelizer");
  cuda_check(cudaMalloc(&dT, sizeof(unsigned int) * (T_.size() + 1)), "Voxelizer");
  cudaMemcpy(dP, P_.data(), sizeof(float) * P_.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(dT, T_.data(), sizeof(unsigned int) * T_.size(), cudaMemcpyHostToDevice);
  gm_ctx* ctx = shared_ctx();
  s = gm_voxelize(ctx, &d, dP, (int64_t)(P_.size() / 3), dT, (int64_t)(T_.size() / 3), grid_.grid_gpu().voxels,
                  nullptr);
  cudaDeviceSynchronize();
  cudaFree(dP);
  cudaFree(dT);
  if (s != GM_OK) throw Grid::Exception(message(ctx, s, "Voxelizer::VoxelizeConservative"));
}

// ------------------------------------------------------------------ GMorpho

GMorpho::GMorpho() {}
GMorpho::~GMorpho() {
  if (ctx_) gm_ctx_destroy(ctx_);
}

void GMorpho::check(int status, const char* what) {
  if (status != GM_OK) throw Exception(message(ctx_, status, what));
}

void GMorpho::Load(const float* P, const float* N, int nv, const unsigned int* T, int nf, int base_res,
                   float se_size) {
  se_size_ = se_size;
  const float margin = se_size_ + 2.f / (2 * (float)base_res);  // GMorpho.cu:7735
  voxelizer_.Load(P, N, nv, T, nf);
  voxelizer_.VoxelizeConservative(base_res, margin);
  const Grid& g = voxelizer_.grid();
  input_grid_.Init(g.bbox_min(), g.bbox_max(), g.res(), g.data_res(), g.cell_size());
  input_grid_.CopyVoxelsFrom(g);
  dilation_grid_.Init(g.bbox_min(), g.bbox_max(), g.res(), g.data_res(), g.cell_size());
  dilation_grid_.CopyVoxelsFrom(input_grid_);
  closing_grid_.Init(g.bbox_min(), g.bbox_max(), g.res(), g.data_res(), g.cell_size());
  closing_grid_.CopyVoxelsFrom(dilation_grid_);
  bbox_ = BoundingBox(g.bbox_min(), g.bbox_max());
  if (!ctx_) {
    int dev = 0;
    cudaGetDevice(&dev);
    check(gm_ctx_create(dev, &ctx_), "gm_ctx_create");
  }
}

void GMorpho::close(const ScaleField* sf, int uniform_radius, int se) {
  if (!ctx_) throw Exception("Load must come first");
  gm_grid_desc d = desc_of(input_grid_);
  check(gm_close(ctx_, &d, input_grid_.grid_gpu().voxels,
                 sf ? reinterpret_cast<const int8_t*>(sf->scale_grid()) : nullptr, uniform_radius, (gm_mode)mode_,
                 (gm_se)se, closing_grid_.grid_gpu().voxels, dilation_grid_.grid_gpu().voxels, nullptr, nullptr),
        "gm_close");
}

void GMorpho::close_rotcube(const ScaleField& sf, const FrameField& ff) {
  if (!ctx_) throw Exception("Load must come first");
  gm_grid_desc d = desc_of(input_grid_);
  const float* q = ff.quats_pong();
  check(gm_close_rotcube(ctx_, &d, input_grid_.grid_gpu().voxels, reinterpret_cast<const int8_t*>(sf.scale_grid()), 0,
                         q, ff.res()[0], (gm_mode)mode_, closing_grid_.grid_gpu().voxels,
                         dilation_grid_.grid_gpu().voxels, nullptr, nullptr),
        "gm_close_rotcube");
}

void GMorpho::Update(Mesh& mesh, const ScaleField& sf, const FrameField& ff) {
  // gate of GMorpho.cu:7783: morphology only when floor(2 gs / cell) > 1;
  // the frame field matters with the asymmetric closing only (:7785-7791)
  if (std::floor(2.f * sf.global_scale() / cell_size()) > 1.f) {
    if (use_asymmetric_closing_ && use_frame_field_)
      close_rotcube(sf, ff);
    else
      close(&sf, 0, use_asymmetric_closing_ ? GM_SE_CUBE : GM_SE_SPHERE);
  } else {
    closing_grid_.CopyVoxelsFrom(input_grid_);
  }
  ExtractClosingMesh(mesh, use_asymmetric_closing_ ? 200 : 20);
}

void GMorpho::DilateBySphereMipmap(const ScaleField& sf) { close(&sf, 0, GM_SE_SPHERE); }
void GMorpho::DilateByCubeMipmap(const ScaleField& sf) { close(&sf, 0, GM_SE_CUBE); }
void GMorpho::DilateByRotCubeMipmap(const ScaleField& sf, const FrameField& ff) { close_rotcube(sf, ff); }
// The closing runs both halves in one call; the erosion of the last
// dilation is already in closing_grid().
void GMorpho::ErodeBySphereMipmap(const ScaleField&) {}

void GMorpho::Update(Mesh& mesh, float se_size) {
  se_size_ = se_size;
  close(nullptr, (int)std::floor(2.f * se_size / cell_size()), GM_SE_CUBE);  // GMorpho.cu:7819-7845
  ExtractClosingMesh(mesh, 20);
}

void GMorpho::DilateByCubeMipmap(float se_size) { close(nullptr, (int)std::floor(2.f * se_size / cell_size()), GM_SE_CUBE); }
void GMorpho::DilateBySphereMipmap(float se_size) {
  close(nullptr, (int)std::floor(2.f * se_size / cell_size()), GM_SE_SPHERE);
}
void GMorpho::ErodeBySphereMipmap(float) {}

void GMorpho::ErodeByBVH(float se_size) {
  if (!ctx_) throw Exception("Load must come first");
  gm_grid_desc d = desc_of(input_grid_);
  check(gm_erode_bvh(ctx_, &d, input_grid_.grid_gpu().voxels, dilation_grid_.grid_gpu().voxels,
                     (int32_t)std::floor(2.f * se_size / cell_size()), closing_grid_.grid_gpu().voxels, nullptr),
        "gm_erode_bvh");
}

void GMorpho::ExtractClosingMesh() { ExtractClosingMesh(morpho_mesh_, 20); }

void GMorpho::ExtractClosingMesh(Mesh& mesh, int iters) {
  gm_grid_desc d = desc_of(closing_grid_);
  gm_mesh_view mv;
  check(gm_mesh(ctx_, &d, closing_grid_.grid_gpu().voxels, bilateral_filtering_ ? iters : 0, &mv, nullptr), "gm_mesh");
  mesh.P().resize((size_t)mv.num_vertices);
  mesh.N().resize((size_t)mv.num_vertices);
  mesh.T().resize((size_t)mv.num_triangles);
  check(gm_mesh_download(ctx_, mv.num_vertices ? &mesh.P()[0][0] : nullptr,
                         mv.num_vertices ? &mesh.N()[0][0] : nullptr, mv.num_triangles ? &mesh.T()[0][0] : nullptr,
                         nullptr),
        "gm_mesh_download");
  if (&mesh != &morpho_mesh_) morpho_mesh_ = mesh;
}

}  // namespace MorphoGraphics

// ------------------------------------------------------------------ MarchingCubesMesher

MarchingCubesMesher::MarchingCubesMesher(Grid* grid) : grid_(grid) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (gm_ctx_create(dev, &ctx_) != GM_OK) ctx_ = nullptr;
}

MarchingCubesMesher::~MarchingCubesMesher() {
  if (ctx_) gm_ctx_destroy(ctx_);
}

void MarchingCubesMesher::createMesh3D(const unsigned char* d_voxels, int iters) {
  if (!ctx_) throw MorphoGraphics::Grid::Exception("MarchingCubesMesher: no context");
  gm_grid_desc d;
  const int res = (int)grid_->getNbCellsX() / 2;
  for (int a = 0; a < 3; a++) {
    d.bbox_min[a] = grid_->getOrigin()[a];
    d.bbox_max[a] = grid_->getOrigin()[a] + 2.f * grid_->getCellSizeX() * res;
    d.data_res[a] = res;
  }
  d.res = res;
  d.cell_size = 2.f * grid_->getCellSizeX();
  gm_mesh_view mv;
  const int s = gm_mesh(ctx_, &d, d_voxels, iters, &mv, nullptr);
  if (s != GM_OK) throw MorphoGraphics::Grid::Exception(message(ctx_, s, "MarchingCubesMesher::createMesh3D"));
  V_ = mv.vertices;
  N_ = mv.normals;
  T_ = mv.triangles;
  nv_ = (unsigned int)mv.num_vertices;
  nt_ = (unsigned int)mv.num_triangles;
}

void MarchingCubesMesher::getDeviceMesh(const float** V, const float** N, unsigned int* VSize,
                                        const unsigned int** T, unsigned int* TSize) const {
  *V = V_;
  *N = N_;
  *VSize = nv_;
  *T = T_;
  *TSize = nt_;
}
