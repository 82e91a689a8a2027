/*
 * gm_oracle.h — CPU oracle for the GMorpho hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C on the host,
 * the algorithms of the reference GMorpho library (superboubek/Broxy,
 * GMorpho/ CUDA sources) so that the CUDA kernels of broxy_gb300 can be checked
 * against it.  Only the test-suite, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py load it.  The product never calls it.
 *
 * Parity status: pinned to the reference itself.  The reference ships no
 * tests, golden vectors or fixtures for this path; its own CUDA morphology
 * and meshing sources are compiled for the GPU (oracle/refbuild/, output in
 * oracle/_ref/) and run through GMorpho::Update on seeded inputs, and its
 * dilation, contour and closing grids equal this restatement's byte for
 * byte, its meshes triangle for triangle (tests/test_oracle_ref.py).  A
 * second, independent transliteration of the reference's float traversal
 * kernels (tests/golden/gen_golden.py) checks it on small grids on the CPU.
 * The frame-field solver (oracle/framefield.py) is the exception: it is not
 * part of the reference build, so its parity stays unpinned.
 *
 * Layouts (same as the reference):
 *   grid   : uint8[res^3], byte c = cx + res*cy + res*res*cz packs the 2x2x2
 *            fine voxels 2c + (i,j,k) at bit i + 2j + 4k (GMorpho/Grid.h:57-64,
 *            GMorpho/Voxelizer.cu:815-823).
 *   scale  : int8[(2res)^3] fine radii, index x + N*y + N*N*z, N = 2 res
 *            (GMorpho/ScaleField.cu:61-72, GMorpho/Grid.cu:985).
 *   pyramid: uint64 texels, level l has (res>>l)^3 texels stored x-fastest,
 *            levels concatenated from 0 (finest) to log2(res) (root).
 */
#ifndef GM_ORACLE_H
#define GM_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

int gmo_version(void);

/* a4 — pyramid texel count and build (GMorpho/Grid.cu:957-998, 733-805). */
int64_t gmo_pyramid_size(int res);
void gmo_pyramid_build(const uint8_t *grid, const int8_t *scale, int res,
                       uint64_t *pyr);

/* a5 / a5c / a7 — dilation predicate at the integer lattice point p
 * (fine units) with structuring radius `radius` (the 7-bit texel radius).
 * se = 0: sphere, test sqd(p, box q) < (radius+1)^2 (GMorpho.cu:2858-2867,
 *          193-210);  se = 1: cube, q in [p-radius-1, p+radius]
 *          (GMorpho.cu:1868-1871, 140-149, 351-363).
 * Hierarchical traversal of the pyramid, as the reference kernels do. */
int gmo_dilate_query(const uint64_t *pyr, int res, int se,
                     int px, int py, int pz, int radius);

/* a9 / a11 — erosion predicate at a point given in half-voxel units
 * (q2 = 2 * point): true iff some occupied voxel q of the pyramid's grid has
 * sqd(point, box q) < (r(q) - 1)^2 (GMorpho.cu:4403-4411, 5283-5349). */
int gmo_erode_query2(const uint64_t *pyr, int res, int qx2, int qy2, int qz2);

/* Same predicates by exhaustive search over the grid (no pyramid). */
int gmo_dilate_query_brute(const uint8_t *grid, const int8_t *scale, int res,
                           int se, int px, int py, int pz, int radius);
int gmo_erode_query2_brute(const uint8_t *grid, const int8_t *scale, int res,
                           int qx2, int qy2, int qz2);

/* a5..a11 — the reference's two-level closing (GMorpho.cu:7775-7817).
 * mode 0 = GM_REF (base pass + contour refinement, bit-exact restatement),
 * mode 1 = GM_EXACT (fine predicates applied at every fine voxel).
 * se = 0 sphere dilation, 1 cube dilation; erosion is always by sphere.
 * Outputs D (dilation), S (dilation contour), C (closing), each res^3 bytes.
 * Any output pointer may be NULL.  Returns 0 on success. */
int gmo_close(const uint8_t *X, const int8_t *scale, int res,
              const int *data_res, int mode, int se,
              uint8_t *D, uint8_t *S, uint8_t *C);

/* gmo_close, also giving the sizes of the reference's two refinement
 * lists in GM_REF: lists[0] = cells tagged by ComputeContourBaseTight on
 * the base dilation (the fine dilation's work list, GMorpho.cu:3573-3590),
 * lists[1] = cells tagged by ComputeContourBase on the base erosion (the
 * persistent erosion kernel's work list, GMorpho.cu:6661-6688). */
int gmo_close_lists(const uint8_t *X, const int8_t *scale, int res,
                    const int *data_res, int mode, int se,
                    uint8_t *D, uint8_t *S, uint8_t *C, int64_t *lists);

/* Pure brute-force ball closing (no pyramid, no two-level structure):
 * the GM_EXACT definition evaluated by exhaustive search.  Small grids only. */
int gmo_close_exact_brute(const uint8_t *X, const int8_t *scale, int res,
                          int se, uint8_t *C);

/* f2 — rotated-cube dilation under a quaternion field Q: (x, y, z, w)
 * floats per node of a qres^3 lattice, x-fastest (FrameField::quats_pong).
 * gmo_rotcube_frame: the rotated axes b_x, b_y, b_z (9 floats) at lattice
 * point i of a grid of `res` points per axis (InterpolateQuaternionField
 * and normalize (conj (quat)), GMorpho.cu:1631-1710, 1735-1745).
 * gmo_rotcube_query: the traversal of DilateByRotCubeByTexMipmap{Base,}
 * with the frame at point p of a frame_res grid, centre c (fine units) and
 * half size `radius`.
 * gmo_close_rotcube: DilateByRotCubeMipmap then the sphere erosion
 * (GMorpho.cu:3058-3230, 7785-7803); mode 0 GM_REF, 1 GM_EXACT (the fine
 * predicate at every fine voxel).  Outputs may be NULL; returns 0. */
void gmo_rotcube_frame(const float *Q, int qres, int ix, int iy, int iz,
                       int res, float *axes);
int gmo_rotcube_query(const uint64_t *pyr, int res, const float *Q, int qres,
                      int px, int py, int pz, int frame_res, int cx, int cy,
                      int cz, int radius);
int gmo_close_rotcube(const uint8_t *X, const int8_t *scale, int res,
                      const int *data_res, const float *Q, int qres, int mode,
                      uint8_t *D, uint8_t *S, uint8_t *C);

/* a12..a15 — contour marching cubes in the reference's emission order.
 * First call with V == NULL to get the counts.  Returns 0 on success,
 * -1 if the capacities are too small. */
int gmo_mc(const uint8_t *C, int res, const float *bbox_min, float cell_size,
           float isovalue, float *V, int64_t v_cap, uint32_t *T, int64_t t_cap,
           int64_t *nv, int64_t *nt);

/* a16 — area-weighted vertex normals then `iters` bilateral normal
 * filtering iterations (GMorpho.cu:6498-6620, 6950-6990), accumulated in
 * triangle order. */
void gmo_normals(const float *V, int64_t nv, const uint32_t *T, int64_t nt,
                 int iters, float *N);

/* a3 — ScaleField (GMorpho/ScaleField.cu:81-146). mode: 1 MAX, 2 MIN, 3 ZERO. */
void gmo_scale_brush(int8_t *scale, int n, const float *bbox_min,
                     float cell_size, const float *pos, float scale_value,
                     float support, float global_scale, int mode);

/* a2 — Voxelizer grid attributes (GMorpho/Voxelizer.cu:431-455). */
void gmo_grid_attributes(const float *P, int64_t nv, int base_res,
                         float margin, float *bbox_min, float *bbox_max,
                         float *cell_size, int *data_res);
/* a2 — conservative surface + parity solid voxelization into the 2x2x2
 * byte grid (res^3 bytes, zeroed by the caller). */
void gmo_voxelize(const float *P, int64_t nv, const uint32_t *T, int64_t nf,
                  int res, const float *bbox_min, float cell_size,
                  uint8_t *grid);

/* Morton code of a base cell, 10 bits per axis, x lowest
 * (GMorpho/cuda_math.h:111-117,148-152). */
uint32_t gmo_morton3(uint32_t x, uint32_t y, uint32_t z);

#ifdef __cplusplus
}
#endif
#endif
