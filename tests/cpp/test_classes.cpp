// Exercises the reference-style C++ classes over libgmorpho_gb300, the way
// the reference viewer drives them (BroxyViewer.cpp:108-232): load a mesh,
// set a global scale, Update, brush the scale field, Update again, then the
// asymmetric closing with and without a frame field.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <cstdlib>
#include <vector>

#include "gmorpho/GMorpho.h"

using namespace MorphoGraphics;

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s in.off out.off [dump_dir]\n", argv[0]);
    return 2;
  }
  Mesh input;
  if (!input.loadOFF(argv[1])) {
    fprintf(stderr, "cannot read %s\n", argv[1]);
    return 2;
  }
  std::vector<float> P, N;
  std::vector<unsigned int> T;
  for (auto& p : input.P()) { P.push_back(p[0]); P.push_back(p[1]); P.push_back(p[2]); N.insert(N.end(), 3, 0.f); }
  for (auto& t : input.T()) { T.push_back(t[0]); T.push_back(t[1]); T.push_back(t[2]); }
  try {
    GMorpho gm;
    gm.Load(P.data(), N.data(), (int)input.P().size(), T.data(), (int)input.T().size(), 64, 0.3f);
    ScaleField sf;
    const unsigned int fr = 2 * gm.res()[0];
    sf.set_global_scale(0.05f);
    sf.Init(gm.bbox_min(), gm.bbox_max(), Vec3ui(fr, fr, fr), 0.5f * gm.cell_size());
    sf.UpdateGridGlobalScale();
    FrameField ff;
    Mesh out;
    gm.Update(out, sf, ff);
    const size_t t1 = out.T().size();
    // brush a bigger radius at the first vertex (BroxyViewer.cpp:667-672)
    sf.AddPoint(input.P()[0], 0.15f, 0.3f);
    sf.UpdateGrid();
    gm.Update(out, sf, ff);
    const size_t t2 = out.T().size();
    gm.set_use_asymmetric_closing(true);
    Mesh asym;
    gm.Update(asym, sf, ff);
    if (!out.storeOFF(argv[2])) return 3;
    printf("%zu %zu %zu %zu\n", out.P().size(), t1, t2, asym.T().size());
    // normals are unit length; a vertex whose face normals cancel gets NaN,
    // as normalize() of a zero vector does in the reference
    for (auto& n : out.N()) {
      const float l = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
      if (l == l && !(std::fabs(l - 1.f) < 1e-3f)) return 4;
    }
    // frame field over the grid's box at res / 16 (BroxyViewer.cpp:141-157),
    // first without constraints, then with one (BroxyViewer.cpp:700-713)
    const int fres = (int)gm.res()[0] / 16;
    ff.Init(gm.bbox_min(), gm.bbox_max(), Vec3i(fres, fres, fres), FrameField::BiHarmonicSystem);
    ff.Generate(false, false);
    gm.set_use_frame_field(true);
    Mesh rot0, rot1;
    gm.Update(rot0, sf, ff);
    ff.AddHardConstrainedPoint(input.P()[0], Vec3f(0.f, 0.f, 0.6f));
    // the point is kept at its lattice node, within sqrt(3) cells of it
    if (ff.GetNumberOfHardConstrainedPoints() != 1 ||
        ff.GetHardConstrainedPointId(input.P()[0], 2.f * ff.cell_size()) != 0)
      return 5;
    ff.Generate(false, true);
    gm.Update(rot1, sf, ff);
    printf("%zu %zu\n", rot0.T().size(), rot1.T().size());
    // the frame-field closing's inputs and result, for a parity check
    // against the CPU oracle (argv[3]: a directory)
    if (argc > 3) {
      const std::string dir = argv[3];
      const size_t cells = (size_t)gm.res()[0] * gm.res()[1] * gm.res()[2];
      auto dump = [&](const std::string& name, const void* dev, size_t bytes) {
        std::vector<unsigned char> h(bytes);
        if (cudaMemcpy(h.data(), dev, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
        FILE* f = fopen((dir + "/" + name).c_str(), "wb");
        if (!f) return false;
        fwrite(h.data(), 1, bytes, f);
        fclose(f);
        return true;
      };
      const size_t fr = (size_t)ff.res()[0] * ff.res()[1] * ff.res()[2];
      if (!dump("input.bin", gm.input_grid().grid_gpu().voxels, cells) ||
          !dump("closing.bin", gm.closing_grid().grid_gpu().voxels, cells) ||
          !dump("scale.bin", sf.scale_grid(), 8 * cells) || !dump("quats.bin", ff.quats_pong(), 16 * fr))
        return 7;
      FILE* f = fopen((dir + "/meta.txt").c_str(), "w");
      if (!f) return 7;
      fprintf(f, "%u %u %u %u %d\n", gm.res()[0], gm.input_grid().data_res()[0], gm.input_grid().data_res()[1],
              gm.input_grid().data_res()[2], ff.res()[0]);
      fclose(f);
    }
    try {
      FrameField lo;
      lo.Init(gm.bbox_min(), gm.bbox_max(), Vec3i(4, 4, 4), FrameField::LocalOptimization);
      return 6;
    } catch (const FrameField::Exception&) {
    }
  } catch (const FrameField::Exception& e) {
    fprintf(stderr, "%s\n", e.msg().c_str());
    return 1;
  } catch (const GMorpho::Exception& e) {
    fprintf(stderr, "%s\n", e.msg().c_str());
    return 1;
  } catch (const Grid::Exception& e) {
    fprintf(stderr, "%s\n", e.msg().c_str());
    return 1;
  }
  return 0;
}
