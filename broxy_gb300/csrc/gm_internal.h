// gm_internal.h — launch interfaces shared by the .cu translation units of
// libgmorpho_gb300 (not part of the public C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/gmorpho_gb300.h"

namespace gm {

// Counts the kernels this library launches (reported by the C ABI so that a
// caller can see that the CUDA path ran) and, when profiling is on, times
// every launch with a pair of CUDA events recorded on its own stream.
struct KernelCounter {
  long long launches = 0;
  bool profiling = false;
  struct Pending {
    const char* name;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  std::map<std::string, std::pair<long long, double>> totals;  // name -> (launches, ms)

  cudaEvent_t start(cudaStream_t st);
  void stop(const char* name, cudaStream_t st, cudaEvent_t a);
  void flush();    // waits for the pending events and accumulates
  void release();  // destroys the event pool
};

// Raises `kernel`'s dynamic shared memory limit to at least `bytes` on the
// current device.  The attribute is per device, so the record of what was
// set is kept per (kernel, device); safe to call from several host threads.
// Needed only above the default 48 KB.
cudaError_t ensure_dynamic_smem(const void* kernel, size_t bytes);

// The error bits kernels of this library recorded on the current device
// (kErrTmaTimeout: a TMA tile wait ran out of polls), cleared when `clear`.
cudaError_t kernel_error_flags(unsigned int* flags, bool clear);

// JSON {"name": {"launches": n, "ms": t}, ...} of the counter's totals;
// returns the bytes needed (with the terminating zero), copies when cap allows
int64_t profile_json(KernelCounter& kc, char* buf, int64_t cap);

#define GM_LAUNCH(kc, name, st, ...)                               \
  do {                                                             \
    cudaEvent_t gm_ev0_ = nullptr;                                 \
    if ((kc) != nullptr && (kc)->profiling) gm_ev0_ = (kc)->start(st); \
    __VA_ARGS__;                                                   \
    if ((kc) != nullptr) (kc)->stop(name, st, gm_ev0_);            \
  } while (0)

// The min-plus passes of many closings, gathered for one persistent
// launch per pass (launch_close in phase mode records into it).
struct DpxGroup;
DpxGroup* dpx_group_new();
void dpx_group_free(DpxGroup* g);
void dpx_group_clear(DpxGroup* g);
int dpx_group_size(const DpxGroup* g);
// Room for `njobs` grids (allocates; not while a stream is being captured).
cudaError_t dpx_group_reserve(DpxGroup* g, int njobs);
// Uploads the recorded grids' pass arguments and launches one kernel whose
// resident blocks pull the tiles of all of them from one work counter.
cudaError_t dpx_group_launch(DpxGroup* g, int sms, cudaStream_t st, KernelCounter* kc);

struct CloseArgs {
  int res = 0;        // base resolution of a cubic grid (a multiple of 16)
  int dims[3] = {0, 0, 0};  // box grid rx, ry, rz (multiples of 16) when dims[0] > 0; res is then unused
  int data_res[3] = {0, 0, 0};  // cells with data (GMorpho/Voxelizer.cu:453-454)
  const uint8_t* X = nullptr;   // input packed grid, res^3
  const int8_t* R = nullptr;    // fine radius grid (2res)^3, or nullptr for uniform_r
  int64_t r_sy = 0, r_sz = 0;  // its y / z strides in bytes when it is a view into a larger field (0: dense)
  const uint8_t* rmap_in = nullptr;  // its 16^3-block radius map when already built (launch_radius_map_dense)
  bool xpass_done = false;  // the dilation's x pass already ran (launch_close_xpass) into the workspace
  bool ypass_done = false;  // and its y pass (launch_close_ypass over slabs covering the grid; sphere only)
  bool zpass_done = false;  // and its z pass (launch_close_zpass over slabs covering the grid; sphere only)
  // The dilation is already in the closing's D (D_out, or the workspace's D:
  // close_ws_dilation); launch_close runs the erosion half only.
  bool dilation_done = false;
  // Cells [roi_lo, roi_hi) where the caller needs the closing (roi_hi[0] == 0:
  // everywhere).  Work that cannot reach them is skipped, and the closing and
  // the optional D / S outputs hold no meaningful values outside them.
  int roi_lo[3] = {0, 0, 0}, roi_hi[3] = {0, 0, 0};
  // Resident squared lattice distance field of the input grid (launch_edt,
  // saturated for a radius bound >= every radius of R), as a view with y / z
  // strides in elements: the sphere dilation is then its per-voxel threshold
  // instead of three passes.
  const uint16_t* edt = nullptr;
  int64_t e_sy = 0, e_sz = 0;
  int uniform_r = 0;            // radius when R == nullptr
  int rmax = 2;                 // upper bound of the clamped radius over the grid
  int mode = 0;                 // 0 = GM_REF, 1 = GM_EXACT
  int se = 0;                   // 0 = sphere dilation, 1 = cube dilation
  uint8_t* C_out = nullptr;     // closing, res^3
  uint8_t* D_out = nullptr;     // optional dilation, res^3
  uint8_t* S_out = nullptr;     // optional dilation contour, res^3
  uint8_t* workspace = nullptr; // close_workspace_bytes(res)
  int num_sms = 0;
  // Phase mode (grouped launches over many grids): phase p >= 0 runs only
  // the kernels between the closing's p-th and (p+1)-th min-plus passes
  // (the ones before the first for p = 0) and records its p-th pass into
  // `group` instead of launching it; close_phases() gives the number of
  // phases.  Not for the radius-clamp fallbacks (rmax > 91) or `edt`.
  int phase = -1;
  DpxGroup* group = nullptr;
};

// Phases of launch_close in phase mode: the min-plus passes + 1.
int close_phases(int mode);
// Whether a closing with this radius bound can run in phase mode.
bool close_phase_ok(int rmax, int se);

size_t close_workspace_bytes(int res);
size_t close_workspace_bytes_box(int rx, int ry, int rz);
cudaError_t launch_close(const CloseArgs& a, cudaStream_t st, KernelCounter* kc);
// The dilation's x pass alone (it reads only the input grid), with the
// saturation of the largest radius, so that it can run before the radius
// field is on the device; launch_close then skips it (xpass_done).
cudaError_t launch_close_xpass(const CloseArgs& a, cudaStream_t st, KernelCounter* kc);
// The sphere dilation's y pass on the cells z0 <= z < z1 alone, after the x
// pass, with a radius bound r_bound for that part only: the largest clamped
// radius within 128 fine voxels (along z) of it.  Its values are read only
// by outputs within r + 1 <= 128 fine voxels, whose thresholds (r + 1)^2 the
// part's saturation (r_bound + 1)^2 covers; the tile windows come from
// a.rmap_in, which must hold that part's blocks.  Slabs covering the grid
// make the y pass of launch_close (ypass_done), so that it can run while
// the radius field is still arriving.
cudaError_t launch_close_ypass(const CloseArgs& a, int z0, int z1, int r_bound, cudaStream_t st, KernelCounter* kc);
// Its z pass (threshold and packing into the dilation) on the cells
// z0 <= z < z1 (multiples of 32: whole output tiles), once the y pass has
// run on the cells within 128 fine voxels of them and their radii are on
// the device; r_bound as for launch_close_ypass (every output tile's own
// radius bound is at most it, so windows and saturation are those of the
// whole-grid pass).
cudaError_t launch_close_zpass(const CloseArgs& a, int z0, int z1, int r_bound, cudaStream_t st, KernelCounter* kc);
cudaError_t launch_contour(const uint8_t* D, uint8_t* S, int res, int exact, cudaStream_t st, KernelCounter* kc);
// Where launch_close keeps the dilation D (a.D_out, or its workspace slot),
// and a scratch region of the workspace that launch_close overwrites only
// after it has started (free for work that runs before it on its stream).
uint8_t* close_ws_dilation(const CloseArgs& a);
uint8_t* close_ws_scratch(const CloseArgs& a, size_t* bytes);
// the workspace's second u16 fine field (2 (2 rx)(2 ry)(2 rz) bytes), which
// launch_edt leaves alone
uint16_t* close_ws_field(const CloseArgs& a);

// ---- rotated-cube dilation under a frame field (rotcube.cu) ----
constexpr int kRotCubeMaxLevels = 12;  // res <= 2048
struct RotCubeArgs {
  int res = 0;                  // power of two
  int data_res[3] = {0, 0, 0};
  const uint8_t* X = nullptr;   // input grid
  const int8_t* R = nullptr;    // fine radius grid, or nullptr for uniform_r
  int uniform_r = 0;
  const float* Q = nullptr;     // quaternions (x, y, z, w) of a qres^3 lattice, x-fastest, 16-byte aligned
  int qres = 0;
  int mode = 0;                 // 0 = GM_REF (base pass + conservative contour), 1 = GM_EXACT (every fine voxel)
  uint8_t* D = nullptr;         // dilation out, res^3
  uint8_t* scratch = nullptr;   // rotcube_scratch_bytes(res)
  // Distance shortcuts (optional): E receives the input grid's squared
  // lattice distance field ((2 res)^3 u16) built by launch_edt in
  // edt_workspace (close_workspace_bytes(res); E and scratch must lie
  // outside the parts launch_edt uses).  rmax: the largest clamped radius.
  uint16_t* E = nullptr;
  uint8_t* edt_workspace = nullptr;
  int rmax = 0;
  int num_sms = 0;
};
size_t rotcube_scratch_bytes(int res);

// ---- frame field: the biharmonic quaternion system (framefield.cu) ----
struct FrameFieldGpu {
  int res = 0;
  float4* quats = nullptr;  // res^3 (x, y, z, w)
  double* vecs = nullptr;   // x, r, p, y, Ap: 4 doubles per node each
  double *x = nullptr, *r = nullptr, *p = nullptr, *y = nullptr, *Ap = nullptr;
  double* part = nullptr;   // block partial sums
  double* sc = nullptr;     // CG scalars
  double* h_sc = nullptr;   // pinned copy of the scalars
  uint8_t* S = nullptr;     // screened (hard-constrained) nodes
  cudaGraphExec_t graph = nullptr;
};
cudaError_t frame_field_alloc(FrameFieldGpu& f, int res);
void frame_field_free(FrameFieldGpu& f);
cudaError_t frame_field_fill(FrameFieldGpu& f, float qx, float qy, float qz, float qw, cudaStream_t st,
                             KernelCounter* kc);
// Solves (L^T L + S) q_k = b_k for the four components; nodes[c] / rhs4[4c..]
// are the constrained nodes (x + res*y + res^2*z) and their quaternions, in
// the order given (the last one on a node wins).  Stops when every
// component's residual is <= tol * |b_k| or after max_iters iterations.
cudaError_t frame_field_solve(FrameFieldGpu& f, const int64_t* nodes, const float* rhs4, int npts, double tol,
                              int max_iters, int* iters_out, cudaStream_t st, KernelCounter* kc);
cudaError_t launch_rotcube_dilation(const RotCubeArgs& a, cudaStream_t st, KernelCounter* kc);
// The squared lattice distance field of a cubic grid: per fine voxel p (u16,
// x-fastest, (2 res)^3), the smallest squared distance from lattice point p
// to an occupied fine voxel box, saturated at (rmax + 1)^2 — what the sphere
// dilation's z pass thresholds.  Workspace: close_workspace_bytes(res).
cudaError_t launch_edt(const uint8_t* X, int res, int rmax, uint8_t* workspace, uint16_t* E, cudaStream_t st,
                       KernelCounter* kc);
cudaError_t launch_rmax(const int8_t* R, int64_t n, int* d_out, int sms, cudaStream_t st, KernelCounter* kc);
// The 16^3-block map of the largest raw radius of a dense field of nx*ny*nz
// fine voxels ((nx/16)(ny/16)(nz/16) bytes), and its largest clamped radius
// into *d_rmax (when given).
cudaError_t launch_radius_map_dense(const int8_t* R, int nx, int ny, int nz, uint8_t* out, int* d_rmax,
                                    cudaStream_t st, KernelCounter* kc);

// ---------------------------------------------------------------- crops
cudaError_t launch_box_copy(const uint8_t* src, int sn, const int s0[3], uint8_t* dst, int dn, const int d0[3],
                            const int ext[3], cudaStream_t st, KernelCounter* kc);
cudaError_t launch_embed(const uint8_t* Cc, int ext, uint8_t* C, int res, cudaStream_t st, KernelCounter* kc);
cudaError_t launch_occ_extent(const uint8_t* X, int res, unsigned* d_out3, int sms, cudaStream_t st,
                              KernelCounter* kc);

// ---------------------------------------------------------------- pyramid
size_t pyramid_texels(int res);
cudaError_t launch_pyramid(const uint8_t* grid, const int8_t* R, int uniform_r, int res, uint64_t* pyr,
                           cudaStream_t st, KernelCounter* kc);

// ---------------------------------------------------------------- mesh
struct MeshArgs {
  int res;              // cubic grid edge (cells), unless dims[0] > 0
  int dims[3] = {0, 0, 0};  // box grid rx, ry, rz (multiples of 16) when dims[0] > 0
  const uint8_t* C;     // closed grid
  float bbox_min[3];
  float cell_size;      // base cell size (fine = cell_size / 2)
  float isovalue;       // 0.95 in the reference (GMorpho.cu:6922)
  int bilateral_iters;  // 20 / 200 / 0
  int num_sms;
  // Crop window (edit server).  gres == 0: the whole grid.  Otherwise the
  // grid is a crop whose cell (0,0,0) is global cell `off`, cubes are tagged
  // only in local cells [tag_lo, tag_hi) (and by the global border rule of
  // gres), triangles come from local cells [emit_lo, emit_hi) only, and
  // vertex positions use global fine coordinates with bbox_min the global
  // grid's.
  int gres = 0;
  int off[3] = {0, 0, 0};
  int tag_lo[3] = {0, 0, 0}, tag_hi[3] = {0, 0, 0};
  int emit_lo[3] = {0, 0, 0}, emit_hi[3] = {0, 0, 0};
  int zero_isolated = 0;  // (0,0,0) normal for vertices no triangle uses
  cudaEvent_t geometry_done = nullptr;  // recorded once vertices and triangles are final (before normals)
  // mesh_emit stops after the vertex normals and the bilateral entries:
  // the caller runs the filtering (mesh_filter_group, several meshes at once)
  bool defer_filter = false;
};

// Device-side mesh buffers, grown on demand by the caller of launch_mesh.
struct MeshBuffers {
  void release();
  float* V = nullptr;       // 3 * v_cap
  float* N = nullptr;       // 3 * v_cap
  float* N2 = nullptr;      // unused (kept for ABI-stable layout of the struct)
  float4* N4a = nullptr;    // v_cap, bilateral ping-pong (16-byte normals)
  float4* N4b = nullptr;    // v_cap
  uint2* ent = nullptr;     // 6 * t_cap: filter records as built, vertex v's from 2 rowptr[v] (a
                            // neighbour and its position term |pa-pb|^2, float bits; the sign bit
                            // set when two incident triangles share the neighbour)
  uint2* rec = nullptr;     // 6 * t_cap: the same records packed, vertex v's at [roff[v], roff[v+1])
  uint32_t* roff = nullptr; // v_cap + 1
  uint32_t* T = nullptr;    // 3 * t_cap
  uint32_t* adj = nullptr;  // 3 * t_cap (vertex -> corner list)
  uint32_t* rowptr = nullptr;  // v_cap + 1
  uint32_t* cursor = nullptr;  // v_cap
  int64_t v_cap = 0, t_cap = 0;
  // per-cell / per-brick scratch
  uint32_t* cell_voff = nullptr;  // res^3
  uint32_t* brick_tot = nullptr;  // 3 * (bricks + 1)
  uint32_t* fix = nullptr;        // case-91 fix list: 1 + 4 * fix_cap
  int64_t cells_cap = 0, bricks_cap = 0;
  int fix_cap = 0;
};

// Phase 1: counts (host-synchronous: returns the vertex/triangle totals).
cudaError_t mesh_count(const MeshArgs& a, MeshBuffers& b, cudaStream_t st, KernelCounter* kc, int64_t* nv,
                       int64_t* nt);
// Split form of mesh_count for callers that overlap several meshes: launch
// the counting and an async copy of the 4 totals into h_tot4, then (after
// the stream is synchronised) size the buffers from them.
cudaError_t mesh_count_launch(const MeshArgs& a, MeshBuffers& b, cudaStream_t st, KernelCounter* kc,
                              uint32_t* h_tot4);
cudaError_t mesh_count_finish(MeshBuffers& b, const uint32_t* tot, int64_t* nv, int64_t* nt);
// The buffers mesh_count_launch needs, allocated now (so that the count can
// be captured in a CUDA graph, where nothing may be allocated).
cudaError_t mesh_prepare_grid(const MeshArgs& a, MeshBuffers& b);
// Allocate up front for meshes of a cubic grid of edge res with up to nv
// vertices and nt triangles (later meshes only grow the buffers further).
cudaError_t mesh_reserve(MeshBuffers& b, int res, int64_t nv, int64_t nt);
// Phase 2: emission into b (capacities must be >= counts).
cudaError_t mesh_emit(const MeshArgs& a, MeshBuffers& b, int64_t nv, int64_t nt, cudaStream_t st,
                      KernelCounter* kc);
// The bilateral filtering of several meshes emitted with defer_filter, one
// launch per iteration over all their vertices; `table` is device memory of
// mesh_filter_table_bytes(n) (the call writes it from `h_table`, pinned host
// memory of the same size).  Results equal mesh_emit's own filtering.
size_t mesh_filter_table_bytes(int n);
cudaError_t mesh_filter_group(MeshBuffers* const* meshes, const int64_t* nv, const int* zero_isolated, int n,
                              int iters, void* table, void* h_table, int sms, cudaStream_t st, KernelCounter* kc);

// ---------------------------------------------------------------- scale field
cudaError_t launch_scale_brush(int8_t* R, int n, const float* bbox_min, float cell_size, const float* pos,
                               float scale, float support, float global_scale, int mode, cudaStream_t st,
                               KernelCounter* kc);

// ---------------------------------------------------------------- voxelizer
cudaError_t launch_voxelize(const float* P, int64_t nv, const uint32_t* T, int64_t nf, int res,
                            const float* bbox_min, float cell_size, uint8_t* grid, uint8_t* scratch_fine,
                            cudaStream_t st, KernelCounter* kc);
size_t voxelize_scratch_bytes(int res);
// dir 0: z-words -> packed grid; dir 1: packed grid -> z-words
cudaError_t launch_layout(int res, const uint32_t* zw, uint8_t* grid, int dir, cudaStream_t st, KernelCounter* kc);

// ---------------------------------------------------------------- batch
void batch_release(void* state);
cudaError_t batch_run(void** state, int n, const gm_batch_item* it, int mode, int se, int bilateral, int lanes_req,
                      gm_mesh_view* meshes, int sms, cudaStream_t st, KernelCounter* kc);
int batch_lanes_tuned(void* state);
// fault injection: the next `count` lane buffer allocations fail as out of memory
void batch_inject_alloc_failures(void** state, int count);

// ---------------------------------------------------------------- BVH
cudaError_t bvh_build(const uint8_t* grid, int res, void** handle, uint32_t* scratch_bricks, int* n_out,
                      cudaStream_t st, KernelCounter* kc);
void bvh_free(void* handle);
cudaError_t bvh_query(const void* handle, const int32_t* q2, int64_t nq, int radius, uint8_t* out, cudaStream_t st,
                      KernelCounter* kc);
cudaError_t bvh_erode(const void* handle, const uint8_t* X, const uint8_t* D, int res, const int* data_res,
                      int radius, uint8_t* C, int* d_overflow, cudaStream_t st, KernelCounter* kc);
int bvh_size(const void* handle);
cudaError_t bvh_keys(const void* handle, uint64_t* out, cudaStream_t st);

}  // namespace gm
