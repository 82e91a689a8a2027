// stubs.cu — definitions that the reference GMorpho.cu names but that its
// morphology and meshing path never calls (the OpenGL voxelizer and the
// frame field's cuSolver/Eigen solver are not part of the reference build).
// Each throws if reached.  TEST INFRASTRUCTURE ONLY.
#include <stdexcept>

#include <GMorpho/GMorpho.h>

namespace {
[[noreturn]] void not_built(const char* what) {
  throw std::runtime_error(std::string("not part of the reference build: ") + what);
}
}  // namespace

namespace MorphoGraphics {
Voxelizer::Voxelizer() {}
Voxelizer::~Voxelizer() {}
void Voxelizer::Load(const float*, const float*, int, const unsigned int*, int) { not_built("Voxelizer::Load"); }
void Voxelizer::VoxelizeConservative(int, float) { not_built("Voxelizer::VoxelizeConservative"); }
}  // namespace MorphoGraphics
