/*
 * gmorpho_gb300.h — C ABI of libgmorpho_gb300, the GB300-native GMorpho.
 *
 * Drop-in boundary for the reference library's hot path
 *   GMorpho::Load -> Voxelizer, ScaleField, GMorpho::Update
 *   (dilation, erosion, marching cubes, normals), Grid pyramids, BVH.
 * Each entry point names the reference interface it replaces
 * (superboubek/Broxy, GMorpho/...).
 *
 * Conventions
 *   - plain pointers and sizes; d_* are device pointers, h_* host pointers;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy stream);
 *   - every call returns a gm_status and never aborts; a message for the
 *     last failure is available from gm_ctx_last_error();
 *   - grids use the reference's packed layout: uint8[res^3], byte
 *     cx + res*cy + res*res*cz holds fine voxels 2c + (i,j,k) at bit
 *     i + 2j + 4k; fine fields (radius grid) are x-fastest with edge 2*res;
 *   - device buffers passed in must be 16-byte aligned;
 *   - res is a power of two in [16, 1024] (fine edge 32 .. 2048).
 */
#ifndef GMORPHO_GB300_H
#define GMORPHO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GM_ABI_VERSION 1

typedef enum {
  GM_OK = 0,
  GM_ERR_INVALID_ARGUMENT = 1,
  GM_ERR_CUDA = 2,
  GM_ERR_OUT_OF_MEMORY = 3,
  GM_ERR_UNSUPPORTED = 4,
  GM_ERR_CAPACITY = 5,
  GM_ERR_NOT_READY = 6
} gm_status;

/* GM_REF reproduces the reference's two-level closing bit for bit;
 * GM_EXACT applies the fine predicates at every voxel (pure ball closing). */
typedef enum { GM_REF = 0, GM_EXACT = 1 } gm_mode;
/* dilation structuring element; the erosion is always by sphere
 * (GMorpho/GMorpho.cu:7784-7790). */
typedef enum { GM_SE_SPHERE = 0, GM_SE_CUBE = 1 } gm_se;
/* ScaleField brush modes (GMorpho/ScaleField.h:33, EditMode). */
typedef enum { GM_BRUSH_MAX = 1, GM_BRUSH_MIN = 2, GM_BRUSH_ZERO = 3 } gm_brush_mode;

typedef struct gm_ctx gm_ctx;

/* Grid attributes (GMorpho/Grid.h:40-58 GridGPU: bbox, res, data_res,
 * cell_size). */
typedef struct {
  float bbox_min[3];
  float bbox_max[3];
  int32_t res;
  int32_t data_res[3];
  float cell_size;
} gm_grid_desc;

/* A mesh resident on the device, owned by the context and valid until the
 * next call that produces a mesh on the same context. */
typedef struct {
  const float* vertices;      /* 3 * num_vertices */
  const float* normals;       /* 3 * num_vertices */
  const uint32_t* triangles;  /* 3 * num_triangles */
  int64_t num_vertices;
  int64_t num_triangles;
} gm_mesh_view;

/* Options of gm_update (GMorpho::set_* setters, GMorpho/GMorpho.h:67-72). */
typedef struct {
  int32_t use_asymmetric_closing; /* 1: cube dilation + 200 bilateral iterations */
  int32_t bilateral_filtering;    /* 0: plain normals */
  int32_t mode;                   /* gm_mode */
} gm_update_opts;

/* ---------------------------------------------------------------- misc */
const char* gm_status_string(gm_status s);
int gm_abi_version(void);

/* Context: device selection, cached workspaces and the last mesh.  Replaces
 * the global GMorpho / Grid / MarchingCubesMesher state of the reference
 * (GMorpho/GMorpho.h:48-170, BroxyViewer.cpp:42-45). */
gm_status gm_ctx_create(int device, gm_ctx** out);
gm_status gm_ctx_destroy(gm_ctx* ctx);
const char* gm_ctx_last_error(const gm_ctx* ctx);
/* number of this library's kernels launched on the context so far */
long long gm_ctx_kernel_launches(const gm_ctx* ctx);
/* Error bits that this library's kernels recorded on the current device
 * instead of trapping: bit 0 = a shared-memory tile load (TMA) was not
 * complete within its poll limit (the results of that call are not
 * trustworthy).  Waits for the device's work; clears the bits when `clear`.
 * No counterpart in the reference (which checks cudaGetLastError only,
 * GMorpho/GMorpho.cu:50-56). */
gm_status gm_kernel_error_flags(uint32_t* flags, int32_t clear);
/* Per-kernel timing (the reference prints GET_TIME spans around each
 * kernel, GMorpho/timing.h:28): when enabled, every launch is bracketed by
 * CUDA events on its own stream.  gm_ctx_profile_read writes a JSON object
 * {kernel: {"launches": n, "ms": total}} into buf and returns the bytes
 * needed (including the terminating zero). */
gm_status gm_ctx_profile(gm_ctx* ctx, int32_t enable);
gm_status gm_ctx_profile_reset(gm_ctx* ctx);
int64_t gm_ctx_profile_read(gm_ctx* ctx, char* buf, int64_t cap);

/* ---------------------------------------------------------------- a2 */
/* Voxelizer::ComputeGridAttributes (GMorpho/Voxelizer.cu:431-455): bbox of
 * the points grown by 2*maxExtent/base_res + margin, cubic res = base_res. */
gm_status gm_grid_attributes(const float* h_points, int64_t num_points, int32_t base_res, float margin,
                             gm_grid_desc* out);
/* Voxelizer::VoxelizeConservative (GMorpho/Voxelizer.cu:724-796): parity
 * solid fill plus conservative surface voxels, into a zeroed packed grid. */
gm_status gm_voxelize(gm_ctx* ctx, const gm_grid_desc* desc, const float* d_points, int64_t num_points,
                      const uint32_t* d_triangles, int64_t num_triangles, uint8_t* d_grid, void* stream);

/* ---------------------------------------------------------------- a3 */
/* ScaleField::UpdateGridGlobalScale (GMorpho/ScaleField.cu:143-146). */
gm_status gm_scalefield_fill(gm_ctx* ctx, int8_t* d_scale, int64_t num_voxels, int32_t value, void* stream);
/* ScaleField::UpdateGrid / UpdateScaleGrid (GMorpho/ScaleField.cu:81-202),
 * one brush point; cell_size is the fine (scale-field) cell size. */
gm_status gm_scalefield_brush(gm_ctx* ctx, int8_t* d_scale, int32_t fine_res, const float* bbox_min,
                              float cell_size, const float* position, float scale, float support,
                              float global_scale, gm_brush_mode mode, void* stream);

/* ---------------------------------------------------------------- a4 */
/* Grid::BuildTexMipmaps(const ScaleField&) (GMorpho/Grid.cu:1000-1154): the
 * OR / max-radius texel pyramid, levels 0..log2(res) concatenated. */
int64_t gm_pyramid_texels(int32_t res);
gm_status gm_pyramid_build(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_grid, const int8_t* d_scale,
                           int32_t uniform_radius, uint64_t* d_pyramid, void* stream);

/* ---------------------------------------------------------------- a5..a11 */
/* GMorpho::DilateBySphereMipmap / DilateByCubeMipmap + ErodeBySphereMipmap
 * (GMorpho/GMorpho.cu:3231-3314, 3538-3596, 6627-6702) on device buffers.
 * d_scale = NULL uses uniform_radius everywhere; radii are clamped to
 * [2,127] (GMorpho/Grid.cu:990-991).  d_dilation / d_contour may be NULL. */
gm_status gm_close(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_input, const int8_t* d_scale,
                   int32_t uniform_radius, gm_mode mode, gm_se se, uint8_t* d_closing, uint8_t* d_dilation,
                   uint8_t* d_contour, void* stream);

/* The closing of gm_close for callers that cannot call cudaMalloc (a host
 * application that owns the device memory budget and forbids library
 * allocations, or a latency-bound loop that cannot take cudaMalloc's
 * implicit synchronisation).  No counterpart in the reference library.
 * Allocates nothing: its scratch is a fixed 16 MiB array held by the library
 * on every GPU that loads it (until exit), so res <= 64 (128^3 fine voxels);
 * larger grids return GM_ERR_CAPACITY.  Inputs and outputs are the caller's,
 * as for gm_close, on the current device.  Every call looks up that array's
 * device address for the current device and context (cudaGetSymbolAddress,
 * which allocates nothing), so a device reset or a context switch between
 * calls is safe.  With a radius field (d_scale != NULL) the call reads the
 * field's radius bound back to the host and so waits for `stream` to drain
 * up to that point; with a uniform radius it only enqueues work.  All calls
 * share the one array and each leaves its contents behind: calls that
 * overlap on the GPU (other streams, other threads) race on it.  No context,
 * no kernel counter, no error message beyond the status. */
gm_status gm_close_noalloc(const gm_grid_desc* desc, const uint8_t* d_input, const int8_t* d_scale,
                           int32_t uniform_radius, gm_mode mode, gm_se se, uint8_t* d_closing,
                           uint8_t* d_dilation, uint8_t* d_contour, void* stream);

/* ---------------------------------------------------------------- frame field */
/* FrameField with the BiHarmonicSystem method (GMorpho/FrameField.h,
 * FrameField.cu, FrameFieldSparseBiharmonic.cu): a quaternion per node of a
 * res^3 lattice over [bbox_min, bbox_max] (cell size = largest extent / res),
 * interpolating up to 20 hard-constrained rotations.  The context must
 * outlive the field. */
typedef struct gm_frame_field gm_frame_field;
gm_status gm_frame_field_create(gm_ctx* ctx, const float* bbox_min, const float* bbox_max, int32_t res,
                                gm_frame_field** out);
gm_status gm_frame_field_destroy(gm_frame_field* ff);
/* AddHardConstrainedPoint(position, twist) (FrameField.cu:64-77): the node
 * floor((position - bbox_min) / cell_size) takes the rotation of rotation
 * vector `twist` (axis * angle).  GM_ERR_CAPACITY past 20 points (the
 * reference ignores them silently); GM_ERR_INVALID_ARGUMENT for a node
 * outside the lattice (the reference writes out of bounds). */
gm_status gm_frame_field_add_point(gm_frame_field* ff, const float* position, const float* twist);
gm_status gm_frame_field_update_point(gm_frame_field* ff, int32_t i, const float* twist);
int32_t gm_frame_field_num_points(const gm_frame_field* ff);
gm_status gm_frame_field_get_point(const gm_frame_field* ff, int32_t i, float* grid_position, float* twist);
/* Generate (FrameField.cu:556-575): without points every node is
 * (0, 1, 0, 0); otherwise, per component k, (L^T L + S) q_k = b_k with L the
 * degree-normalised 6-neighbour Laplacian (float entries as the reference
 * builds them), S the indicator of constrained nodes and b_k their
 * quaternions (sin(theta/2) axis, cos(theta/2)).  The reference factors the
 * system in float (sparse Cholesky); here conjugate gradients in double
 * until every residual is below 1e-10 |b_k|.  *iterations (may be NULL): the
 * iterations run.  Synchronises the stream. */
gm_status gm_frame_field_generate(gm_frame_field* ff, int32_t* iterations, void* stream);
/* The device quaternions ((x, y, z, w) floats per node, x-fastest; the
 * reference's quats_pong), valid until the next generate or destroy. */
gm_status gm_frame_field_quats(const gm_frame_field* ff, const float** d_quats, int32_t* res);
/* FrameField::RotationToTwistCayley (FrameField.cu:228-252) in double;
 * GM_ERR_INVALID_ARGUMENT for half turns (R + I singular). */
gm_status gm_rotation_to_twist(const float* e_x, const float* e_y, const float* e_z, float* twist);

/* GMorpho::Update with use_frame_field (GMorpho/GMorpho.cu:7785-7803):
 * DilateByRotCubeMipmap (GMorpho.cu:3058-3230, 1712-1837, 2464-2602), the
 * dilation by cubes of half size r(p) rotated by the quaternion field
 * interpolated at p, then ErodeBySphereMipmap as in gm_close.  d_quats:
 * (x, y, z, w) floats per node of a quat_res^3 lattice, x-fastest, 16-byte
 * aligned (FrameField::quats_pong, e.g. gm_frame_field_quats).  GM_REF: the
 * reference's base pass over cells inside data_res and its conservative
 * contour refinement; GM_EXACT: the per-voxel predicate everywhere.  The
 * reference reads one node past the field on its top faces; those reads
 * are clamped to the last node here. */
gm_status gm_close_rotcube(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_input, const int8_t* d_scale,
                           int32_t uniform_radius, const float* d_quats, int32_t quat_res, gm_mode mode,
                           uint8_t* d_closing, uint8_t* d_dilation, uint8_t* d_contour, void* stream);

/* Grid::TransformToContour (GMorpho/Grid.cu:2381-2408, 1230-1327): fine
 * voxels outside the grid's set that are 6-adjacent to it; GM_REF keeps the
 * reference's restriction to cells in [1, res-2]^3 whose byte is not 0xff,
 * GM_EXACT covers the whole grid.  d_out may equal d_grid. */
gm_status gm_contour(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_grid, uint8_t* d_out, gm_mode mode,
                     void* stream);

/* ---------------------------------------------------------------- a12..a16 */
/* GMorpho::ExtractClosingMesh (GMorpho/GMorpho.cu:6814-7001): contour
 * marching cubes at isovalue 0.95 in the reference's emission order, then
 * normals and `bilateral_iters` bilateral normal iterations. */
gm_status gm_mesh(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_closing, int32_t bilateral_iters,
                  gm_mesh_view* out, void* stream);

/* ---------------------------------------------------------------- a17 */
/* GMorpho::Update(Mesh&, const ScaleField&, const FrameField&)
 * (GMorpho/GMorpho.cu:7775-7817) from host buffers: copies the input grid
 * (and the scale grid when h_scale != NULL) to the device, closes (skipped
 * when floor(2*global_scale/cell_size) <= 1, GMorpho.cu:7783), meshes, and
 * leaves the mesh on the context; fetch it with gm_mesh_download. */
gm_status gm_update(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* h_input, const int8_t* h_scale,
                    float global_scale, const gm_update_opts* opts, int64_t* num_vertices,
                    int64_t* num_triangles, void* stream);
/* Copy the context's last mesh to host buffers (GMorpho.cu:6992-7000);
 * any pointer may be NULL to skip that array. */
/* gm_update that also brings the mesh into the caller's host buffers (3
 * floats per vertex for h_V / h_N, 3 indices per triangle; any may be NULL),
 * overlapping the copies with the work: the dilation's first pass runs
 * while the radius field is uploaded, and vertices and triangles come down
 * while the normals are filtered.  When the mesh exceeds the capacities,
 * GM_ERR_CAPACITY is returned with the counts set and the mesh kept on the
 * device (gm_mesh_download fetches it into larger buffers). */
gm_status gm_update_to_host(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* h_input, const int8_t* h_scale,
                            float global_scale, const gm_update_opts* opts, float* h_V, float* h_N, uint32_t* h_T,
                            int64_t vertex_capacity, int64_t triangle_capacity, int64_t* num_vertices,
                            int64_t* num_triangles, void* stream);
gm_status gm_mesh_download(gm_ctx* ctx, float* h_vertices, float* h_normals, uint32_t* h_triangles, void* stream);

/* ---------------------------------------------------------------- batch */
/* One instance of a batched closing: its own grid, radius and output. */
typedef struct {
  gm_grid_desc desc;
  const uint8_t* d_input;
  const int8_t* d_scale;   /* NULL: uniform_radius */
  int32_t uniform_radius;
  uint8_t* d_closing;      /* output, desc.res^3 bytes */
} gm_batch_item;

/* Batched form of GMorpho::Update for n independent grids of uneven sizes
 * (no reference counterpart: the reference closes one grid per call).
 * lanes > 0: the instances' closings run concurrently on that many internal
 * streams.  lanes = GM_BATCH_GROUPED: the closings go pass by pass, each
 * min-plus pass of all the instances as one persistent launch whose blocks
 * pull the tiles of every instance from one work counter (the kernels
 * between passes per instance on four streams; every instance keeps its
 * own workspace meanwhile; radius bounds <= 91 only, else
 * GM_ERR_INVALID_ARGUMENT).  lanes = 0: the form is autotuned (1, 2, 4, 8,
 * 16 lanes and the grouped form, timed on the first call of a batch
 * signature) and cached.  A uniform-radius batch replays its closing phase
 * as one CUDA graph while the batch is unchanged.  When meshes != NULL
 * every closing is meshed (bilateral_iters iterations) and meshes[i] views
 * device buffers owned by the context until the next batch.  Results equal
 * n separate gm_close + gm_mesh calls bit for bit, in every form. */
#define GM_BATCH_GROUPED (-1)
gm_status gm_batch_close_mesh(gm_ctx* ctx, int32_t n, const gm_batch_item* items, gm_mode mode, gm_se se,
                              int32_t bilateral_iters, int32_t lanes, gm_mesh_view* meshes, void* stream);
/* Form the autotuner chose for the last tuned batch: a lane count, or
 * GM_BATCH_GROUPED (0: none yet). */
int32_t gm_batch_lanes(gm_ctx* ctx);
/* Fault injection for tests: the next `count` lane buffer allocations of
 * gm_batch_close_mesh on this context fail as if the device were out of
 * memory (the call returns GM_ERR_OUT_OF_MEMORY; the context stays usable). */
gm_status gm_batch_inject_alloc_failures(gm_ctx* ctx, int32_t count);

/* ---------------------------------------------------------------- serving */
/* Resident-grid edit server (no reference counterpart: the reference
 * re-closes and re-meshes the whole grid after each brush event,
 * BroxyViewer.cpp:667-672).  An edit is one ScaleField brush point
 * (ScaleField::UpdateGrid, GMorpho/ScaleField.cu:81-141) applied to the
 * resident radius field, followed by an exact LOCAL re-closing of the
 * region it can change and a re-mesh of that region.  Edits are admitted as
 * slots free up (continuous batching); edits whose regions overlap an edit
 * still on the GPU are queued behind it on the GPU (stream order), disjoint
 * edits run concurrently.  The server uses the current device; all calls
 * come from one host thread. */
typedef struct gm_server gm_server;

typedef struct {
  int32_t slots;            /* concurrent edits (1..16) */
  int32_t max_crop_res;     /* largest local re-closing, base cells per axis (a multiple of 16, or res) */
  int32_t rmax;             /* radius bound (fine voxels) for edits and field */
  int32_t mode;             /* gm_mode of the closing */
  int32_t bilateral_iters;  /* normal filtering of the re-meshed patches */
} gm_server_opts;

typedef struct {
  float center[3];     /* brush position (world) */
  float scale;         /* ScalePoint::scale (world): target radius * fine cell, and the brush core */
  float support;       /* ScalePoint::support (world) */
  float global_scale;  /* ScaleField::global_scale, used by GM_BRUSH_ZERO */
  int32_t mode;        /* gm_brush_mode */
} gm_edit;

typedef struct {
  uint64_t ticket;
  int32_t status;          /* GM_OK, GM_ERR_CAPACITY (crop or radius bound), GM_ERR_OUT_OF_MEMORY
                            * (crop buffers larger than the budget, or an allocation failed and the
                            * request timed out), GM_ERR_NOT_READY (timed out waiting), GM_ERR_CUDA */
  float latency_ms;        /* submit -> result, host clock */
  float device_ms;         /* GPU time of the edit */
  int32_t dirty_lo[3];     /* fine-voxel box whose closing was recomputed */
  int32_t dirty_hi[3];
  int32_t crop_res;        /* edge (base cells) of the crop that was re-closed */
  /* mesh of the dirty box (device, valid until the next gm_server_poll): the
   * triangles the whole grid's mesh has in these cells, with bit-identical
   * vertex positions; vertices no patch triangle uses get a zero normal */
  gm_mesh_view patch;
} gm_edit_result;

/* d_input and d_scale stay owned by the caller and must outlive the server;
 * the server edits d_scale in place and keeps its own closed grid. */
gm_status gm_server_create(const gm_grid_desc* desc, const uint8_t* d_input, int8_t* d_scale,
                           const gm_server_opts* opts, gm_server** out);
gm_status gm_server_destroy(gm_server* srv);
gm_status gm_server_submit(gm_server* srv, const gm_edit* edit, uint64_t* ticket);
/* Advances dispatch and returns up to cap finished edits. */
gm_status gm_server_poll(gm_server* srv, gm_edit_result* results, int32_t cap, int32_t* count);
/* Edits queued or on the GPU. */
int32_t gm_server_pending(gm_server* srv);
/* The resident closed grid (device, res^3 bytes). */
const uint8_t* gm_server_closing(gm_server* srv);
long long gm_server_kernel_launches(gm_server* srv);
/* Snapshot / restore of the resident state (the closed grid, res^3 bytes,
 * and the radius field, (2 res)^3 bytes) through host buffers; either
 * snapshot buffer may be NULL.  Both need an idle server (no edit queued or
 * on the GPU: GM_ERR_NOT_READY otherwise).  The input grid stays the
 * caller's.  A restored field above the server's radius bound is copied but
 * answered with GM_ERR_CAPACITY. */
gm_status gm_server_snapshot(gm_server* srv, uint8_t* h_closing, int8_t* h_scale);
gm_status gm_server_restore(gm_server* srv, const uint8_t* h_closing, const int8_t* h_scale);
/* Admission (no reference counterpart).  An edit's crop buffers are taken
 * from a device memory pool when it is dispatched and returned when its
 * result is collected; it is dispatched only while the crop buffers of the
 * edits on the GPU plus its own fit `budget_bytes` (default: the device's
 * free memory at creation less a reserve of max(1 GiB, 5%), capped at the
 * slots' needs for the largest crop; <= 0 keeps the current budget).  An
 * edit waiting in the queue longer than `timeout_ms` (0: no limit) is
 * answered with GM_ERR_NOT_READY, or GM_ERR_OUT_OF_MEMORY when an
 * allocation for it failed. */
gm_status gm_server_set_admission(gm_server* srv, int64_t budget_bytes, float timeout_ms);
/* Bytes of crop buffers of the edits on the GPU, and the budget. */
gm_status gm_server_memory(gm_server* srv, int64_t* inflight_bytes, int64_t* budget_bytes);
/* Fault injection for tests: the next `count` crop-buffer allocations fail
 * as if the device were out of memory (host side; no GPU fault). */
gm_status gm_server_inject_alloc_failures(gm_server* srv, int32_t count);
/* Per-kernel device time of the server's launches (CUDA events around each
 * launch on its slot stream), same JSON form as gm_ctx_profile_read. */
gm_status gm_server_profile(gm_server* srv, int32_t enable);
int64_t gm_server_profile_read(gm_server* srv, char* buf, int64_t cap);

/* ---------------------------------------------------------------- boxes
 * Grids that are boxes of rx * ry * rz base cells (each a multiple of 16),
 * x-fastest, packed like gm_grid_desc grids: a slab of a larger grid on one
 * GPU, a crop, or an instance whose edges are not powers of two.  The
 * closing is the same algorithm with the box's own border (cells outside
 * [1, dims-2] are never contour cells); a box cut out of a larger grid with
 * a margin of rmax + 8 cells on each cut side is exact on its interior. */
typedef struct {
  float bbox_min[3];    /* world position of the box's cell (0,0,0) corner */
  float cell_size;      /* base cell edge */
  int32_t dims[3];      /* rx, ry, rz */
  int32_t data_res[3];  /* cells with data (<= dims) */
} gm_box_desc;

gm_status gm_close_box(gm_ctx* ctx, const gm_box_desc* box, const uint8_t* d_input, const int8_t* d_scale,
                       int32_t uniform_radius, gm_mode mode, gm_se se, uint8_t* d_closing, void* stream);

/* The closing of a box on the cells [roi_lo, roi_hi) only (no reference
 * counterpart: a local re-closing after an edit, or a slab's owned cells).
 * Those cells are bit-identical to gm_close_box's; d_closing holds
 * unspecified bytes elsewhere.  Passes skip the tiles that cannot reach the
 * region (the dilation within its erosion and dilation reach). */
gm_status gm_close_box_region(gm_ctx* ctx, const gm_box_desc* box, const uint8_t* d_input, const int8_t* d_scale,
                              int32_t uniform_radius, gm_mode mode, gm_se se, const int32_t roi_lo[3],
                              const int32_t roi_hi[3], uint8_t* d_closing, void* stream);

/* Where a box sits in a cubic global grid, and which of its cells to mesh:
 * triangles of cells [emit_lo, emit_hi), the global grid's border rule and
 * global vertex coordinates (box->bbox_min must then be the GLOBAL grid's
 * corner), so that the meshes of adjacent windows hold exactly the global
 * mesh's triangles.  Vertices no triangle of the window uses (one layer past
 * emit_hi) get a zero normal. */
typedef struct {
  int32_t origin[3];    /* global cell of the box's cell (0,0,0) */
  int32_t global_res;
  int32_t emit_lo[3], emit_hi[3];
} gm_mesh_window;

/* Mesh of a closed box (win NULL: the whole box, its own border rule). */
gm_status gm_mesh_box(gm_ctx* ctx, const gm_box_desc* box, const uint8_t* d_closing, const gm_mesh_window* win,
                      int32_t bilateral_iters, gm_mesh_view* out, void* stream);

/* Host mesh file output, format by extension: ".off" (the reference's
 * Mesh::storeOFF text form, Common/Mesh.h:627-637), ".pn" (float32
 * position + normal per vertex, the reference's PN form) or ".ply" (binary
 * little-endian: float x y z nx ny nz, uchar-count uint faces).  N may be
 * NULL for OFF.  With drop_unused, vertices no triangle uses are left out
 * (indices renumbered), as for a served patch. */
gm_status gm_mesh_store(const char* path, const float* V, const float* N, int64_t nv, const uint32_t* T, int64_t nt,
                        int32_t drop_unused);

/* ---------------------------------------------------------------- a18 */
/* BVH over the set fine voxels of a packed grid (BVH::BuildFromSEList,
 * GMorpho/BVH.cu:661-739): Morton-ordered leaves, radix tree, bottom-up
 * integer boxes.  The handle owns device memory until gm_bvh_destroy. */
typedef struct gm_bvh gm_bvh;
gm_status gm_bvh_build(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_sites, gm_bvh** out,
                       int64_t* num_leaves, void* stream);
gm_status gm_bvh_destroy(gm_bvh* bvh);
/* For each query point (3 int32 per point, in half-voxel units: the centre
 * of fine voxel p is 2p+1), hit = 1 when a leaf voxel centre is at distance
 * < radius (fine voxels) — the leaf test of ErodeBySphereDynamicStack
 * (GMorpho/GMorpho.cu:8957-9060), exact. */
gm_status gm_bvh_query(gm_ctx* ctx, const gm_bvh* bvh, const int32_t* d_points2, int64_t num_points,
                       int32_t radius, uint8_t* d_hits, void* stream);
/* The leaves' 64-bit Morton keys (x in bit 0), ascending. */
gm_status gm_bvh_leaves(gm_ctx* ctx, const gm_bvh* bvh, uint64_t* d_keys, void* stream);
/* GMorpho::ErodeByBVH (GMorpho/GMorpho.cu:9308-9401): builds the BVH of the
 * dilation's contour (TransformToContour) and removes every voxel of D, in
 * cells with D != 0 and X != 0xff inside data_res, whose centre is within
 * distance < radius of a contour voxel centre. */
gm_status gm_erode_bvh(gm_ctx* ctx, const gm_grid_desc* desc, const uint8_t* d_input, const uint8_t* d_dilation,
                       int32_t radius, uint8_t* d_closing, void* stream);

/* ---------------------------------------------------------------- layout */
/* Voxelizer::ConvertBucketToPacketGrid (GMorpho/Voxelizer.cu:798-849):
 * z-words (uint32 of 32 consecutive z voxels, x-fastest over (N, N, N/32))
 * to the packed byte grid, and back. */
gm_status gm_layout_zwords_to_packed(gm_ctx* ctx, int32_t res, const uint32_t* d_zwords, uint8_t* d_grid,
                                     void* stream);
gm_status gm_layout_packed_to_zwords(gm_ctx* ctx, int32_t res, const uint8_t* d_grid, uint32_t* d_zwords,
                                     void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GMORPHO_GB300_H */
