/*
 * gm_oracle.c — CPU restatement of the reference GMorpho hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see gm_oracle.h).  Every function cites the
 * reference file:line it follows.  Integer arithmetic replaces the
 * reference's float predicates: those compare squared distances between
 * power-of-two-scaled integer coordinates and are exact in float, so the
 * integer restatement gives the same booleans (checked by the tests against
 * a float transliteration).  Compiled with -ffp-contract=off; where the
 * reference's nvcc build contracts a multiply-add, fmaf() is written out.
 */
#include "gm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../broxy_gb300/csrc/mc_tables.inc"

int gmo_version(void) { return 1; }

/* ------------------------------------------------------------------ */
/* helpers                                                             */
/* ------------------------------------------------------------------ */

static int ilog2i(int v) {
  int l = 0;
  while ((1 << l) < v) l++;
  return l;
}

/* FillLevel0 clamps the char radius to [2,127] (GMorpho/Grid.cu:990-991). */
static inline int clamp_radius(int s) { return s < 2 ? 2 : (s > 127 ? 127 : s); }

static inline int64_t fine_index(int x, int y, int z, int n) {
  return (int64_t)x + (int64_t)n * y + (int64_t)n * n * z;
}

static inline int grid_bit(const uint8_t *g, int res, int x, int y, int z) {
  int64_t c = (int64_t)(x >> 1) + (int64_t)res * (y >> 1) + (int64_t)res * res * (z >> 1);
  return (g[c] >> ((x & 1) | ((y & 1) << 1) | ((z & 1) << 2))) & 1;
}

/* Morton code, x in bit 0 (GMorpho/cuda_math.h:111-117, 148-152). */
static uint32_t spread3(uint32_t v) {
  uint32_t r = 0;
  for (int b = 0; b < 10; b++) r |= ((v >> b) & 1u) << (3 * b);
  return r;
}
uint32_t gmo_morton3(uint32_t x, uint32_t y, uint32_t z) {
  return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}
static uint32_t compact3(uint32_t m) {
  uint32_t r = 0;
  for (int b = 0; b < 10; b++) r |= ((m >> (3 * b)) & 1u) << b;
  return r;
}

/* ------------------------------------------------------------------ */
/* a4 — texel pyramid                                                  */
/* ------------------------------------------------------------------ */

int64_t gmo_pyramid_size(int res) {
  int64_t t = 0;
  for (int n = res; n >= 1; n >>= 1) t += (int64_t)n * n * n;
  return t;
}

static int64_t level_offset(int res, int level) {
  int64_t t = 0;
  for (int l = 0; l < level; l++) {
    int64_t n = res >> l;
    t += n * n * n;
  }
  return t;
}

/* Level 0: occupancy byte in bits 56..63, radius of child k in bits
 * 7k..7k+6 (GMorpho/Grid.cu:957-998).  Level l+1: bit 56+k = child k has any
 * occupancy, radius field k = max of child k's eight radius fields, counted
 * whether or not the child is occupied (GMorpho/Grid.cu:733-805). */
void gmo_pyramid_build(const uint8_t *grid, const int8_t *scale, int res,
                       uint64_t *pyr) {
  const int n = 2 * res;
  const int levels = ilog2i(res) + 1;
#pragma omp parallel for schedule(static)
  for (int cz = 0; cz < res; cz++)
    for (int cy = 0; cy < res; cy++)
      for (int cx = 0; cx < res; cx++) {
        int64_t c = (int64_t)cx + (int64_t)res * cy + (int64_t)res * res * cz;
        uint64_t t = grid[c];
        for (int k = 7; k >= 0; k--) {
          int fx = 2 * cx + (k & 1), fy = 2 * cy + ((k >> 1) & 1), fz = 2 * cz + (k >> 2);
          int r = clamp_radius(scale[fine_index(fx, fy, fz, n)]);
          t = (t << 7) | (uint64_t)(r & 0x7f);
        }
        pyr[c] = t;
      }
  for (int l = 1; l < levels; l++) {
    const int nf = res >> (l - 1), nt = res >> l;
    const uint64_t *from = pyr + level_offset(res, l - 1);
    uint64_t *to = pyr + level_offset(res, l);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nt; z++)
      for (int y = 0; y < nt; y++)
        for (int x = 0; x < nt; x++) {
          uint64_t out = 0, occ = 0;
          for (int k = 7; k >= 0; k--) {
            int cx = 2 * x + (k & 1), cy = 2 * y + ((k >> 1) & 1), cz = 2 * z + (k >> 2);
            uint64_t v = from[(int64_t)cx + (int64_t)nf * cy + (int64_t)nf * nf * cz];
            int m = 0;
            for (int j = 0; j < 8; j++) {
              int rj = (int)((v >> (7 * j)) & 0x7f);
              if (rj > m) m = rj;
            }
            out = (out << 7) | (uint64_t)m;
            if ((v >> 56) != 0) occ |= 1ull << k;
          }
          to[(int64_t)x + (int64_t)nt * y + (int64_t)nt * nt * z] = out | (occ << 56);
        }
  }
}

/* ------------------------------------------------------------------ */
/* a5 / a5c / a7 / a9 / a11 — pyramid traversals                       */
/* ------------------------------------------------------------------ */

/* squared distance from integer point q to the closed interval [lo, hi] */
static inline int64_t axis_sqd(int64_t q, int64_t lo, int64_t hi) {
  if (q < lo) return (lo - q) * (lo - q);
  if (q > hi) return (q - hi) * (q - hi);
  return 0;
}

typedef struct { int d, x, y, z; } node_t;

/* Depth-first traversal from the root: a node of depth d reads the texel of
 * level (max_depth - d - 1) and tests its eight children (depth d+1, edge
 * N >> (d+1) fine voxels); leaves are fine voxels (GMorpho.cu:2880-2922). */
int gmo_dilate_query(const uint64_t *pyr, int res, int se, int px, int py,
                     int pz, int radius) {
  const int N = 2 * res, L = ilog2i(res), maxd = L + 1;
  const int64_t R = (int64_t)radius + 1; /* "Safety Measure" radius++ (GMorpho.cu:2864) */
  node_t stack[8 * 24];
  int sp = 0;
  stack[sp++] = (node_t){0, 0, 0, 0};
  while (sp > 0) {
    node_t nd = stack[--sp];
    const int level = L - nd.d, nl = res >> level;
    const uint64_t tex = pyr[level_offset(res, level) + (int64_t)nd.x +
                             (int64_t)nl * nd.y + (int64_t)nl * nl * nd.z];
    const int occ = (int)(tex >> 56);
    const int64_t cs = N >> (nd.d + 1);
    for (int k = 0; k < 8; k++) {
      if (!(occ & (1 << k))) continue;
      int bx = 2 * nd.x + (k & 1), by = 2 * nd.y + ((k >> 1) & 1), bz = 2 * nd.z + (k >> 2);
      int64_t lx = bx * cs, ly = by * cs, lz = bz * cs;
      int hit;
      if (se == 0) {
        int64_t s = axis_sqd(px, lx, lx + cs) + axis_sqd(py, ly, ly + cs) + axis_sqd(pz, lz, lz + cs);
        hit = s < R * R;
      } else {
        /* closed AABB overlap of [p - r, p + r] and the node box (GMorpho.cu:140-149) */
        int64_t r = radius;
        hit = (px - r <= lx + cs && px + r >= lx) && (py - r <= ly + cs && py + r >= ly) &&
              (pz - r <= lz + cs && pz + r >= lz);
      }
      if (!hit) continue;
      if (nd.d + 1 == maxd) return 1;
      stack[sp++] = (node_t){nd.d + 1, bx, by, bz};
    }
  }
  return 0;
}

/* Erosion traversal: the threshold of child k is (r_k - 1)^2 with r_k the
 * child's radius field, i.e. the subtree maximum (GMorpho.cu:4412-4425).
 * Coordinates are doubled so that voxel centres are integers. */
int gmo_erode_query2(const uint64_t *pyr, int res, int qx2, int qy2, int qz2) {
  const int N = 2 * res, L = ilog2i(res), maxd = L + 1;
  node_t stack[8 * 24];
  int sp = 0;
  stack[sp++] = (node_t){0, 0, 0, 0};
  while (sp > 0) {
    node_t nd = stack[--sp];
    const int level = L - nd.d, nl = res >> level;
    const uint64_t tex = pyr[level_offset(res, level) + (int64_t)nd.x +
                             (int64_t)nl * nd.y + (int64_t)nl * nl * nd.z];
    const int occ = (int)(tex >> 56);
    const int64_t cs2 = 2 * (int64_t)(N >> (nd.d + 1));
    for (int k = 0; k < 8; k++) {
      if (!(occ & (1 << k))) continue;
      int64_t rk = (int64_t)((tex >> (7 * k)) & 0x7f) - 1;
      int bx = 2 * nd.x + (k & 1), by = 2 * nd.y + ((k >> 1) & 1), bz = 2 * nd.z + (k >> 2);
      int64_t lx = bx * cs2, ly = by * cs2, lz = bz * cs2;
      int64_t s = axis_sqd(qx2, lx, lx + cs2) + axis_sqd(qy2, ly, ly + cs2) + axis_sqd(qz2, lz, lz + cs2);
      if (!(s < 4 * rk * rk)) continue;
      if (nd.d + 1 == maxd) return 1;
      stack[sp++] = (node_t){nd.d + 1, bx, by, bz};
    }
  }
  return 0;
}

int gmo_dilate_query_brute(const uint8_t *grid, const int8_t *scale, int res,
                           int se, int px, int py, int pz, int radius) {
  (void)scale;
  const int N = 2 * res;
  const int64_t R = (int64_t)radius + 1;
  for (int z = 0; z < N; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) {
        if (!grid_bit(grid, res, x, y, z)) continue;
        int hit;
        if (se == 0) {
          int64_t s = axis_sqd(px, x, x + 1) + axis_sqd(py, y, y + 1) + axis_sqd(pz, z, z + 1);
          hit = s < R * R;
        } else {
          hit = (px - radius <= x + 1 && px + radius >= x) && (py - radius <= y + 1 && py + radius >= y) &&
                (pz - radius <= z + 1 && pz + radius >= z);
        }
        if (hit) return 1;
      }
  return 0;
}

int gmo_erode_query2_brute(const uint8_t *grid, const int8_t *scale, int res,
                           int qx2, int qy2, int qz2) {
  const int N = 2 * res;
  for (int z = 0; z < N; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) {
        if (!grid_bit(grid, res, x, y, z)) continue;
        int64_t rk = clamp_radius(scale[fine_index(x, y, z, N)]) - 1;
        int64_t s = axis_sqd(qx2, 2 * x, 2 * x + 2) + axis_sqd(qy2, 2 * y, 2 * y + 2) +
                    axis_sqd(qz2, 2 * z, 2 * z + 2);
        if (s < 4 * rk * rk) return 1;
      }
  return 0;
}

/* ------------------------------------------------------------------ */
/* a6 / a8 / a10 — cell taggers                                        */
/* ------------------------------------------------------------------ */

/* TagVoxelsContourBaseTight: forward 2x2x2 block of cells mixes full (0xff)
 * and non-full cells, c in [0, res-2]^3 (GMorpho/Grid.cu:1572-1608). */
static int tag_tight(const uint8_t *g, int res, int x, int y, int z) {
  if (x > res - 2 || y > res - 2 || z > res - 2) return 0;
  int full = 0;
  for (int k = 0; k < 8; k++) {
    int64_t c = (int64_t)(x + (k & 1)) + (int64_t)res * (y + ((k >> 1) & 1)) +
                (int64_t)res * res * (z + (k >> 2));
    full += g[c] == 0xff;
  }
  return full != 0 && full != 8;
}

/* TagVoxelsContourBase: byte differs from one of its six neighbours,
 * c in [1, res-2]^3 (GMorpho/Grid.cu:1499-1570). */
static int tag_base(const uint8_t *g, int res, int x, int y, int z) {
  if (x < 1 || y < 1 || z < 1 || x > res - 2 || y > res - 2 || z > res - 2) return 0;
  const int64_t s1 = res, s2 = (int64_t)res * res;
  const int64_t c = x + s1 * y + s2 * z;
  const uint8_t v = g[c];
  return g[c - 1] != v || g[c + 1] != v || g[c - s1] != v || g[c + s1] != v ||
         g[c - s2] != v || g[c + s2] != v;
}

/* TagVoxelsContourByErosion: fine voxels outside the dilation that are
 * 6-adjacent to it, for cells c in [1, res-2]^3 whose byte is not 0xff
 * (GMorpho/Grid.cu:1230-1327, 2381-2408). */
static uint8_t contour_byte(const uint8_t *D, int res, int x, int y, int z) {
  if (x < 1 || y < 1 || z < 1 || x > res - 2 || y > res - 2 || z > res - 2) return 0;
  const int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
  const uint8_t center = D[c];
  if (center == 0xff) return 0;
  uint8_t tag = 0;
  for (int k = 0; k < 8; k++) {
    const int ix = k & 1, iy = (k >> 1) & 1, iz = k >> 2;
    /* fine voxel f = 2c + (ix,iy,iz); its 6 neighbours */
    for (int a = 0; a < 6; a++) {
      int dx = a == 0 ? 1 : a == 1 ? -1 : 0;
      int dy = a == 2 ? 1 : a == 3 ? -1 : 0;
      int dz = a == 4 ? 1 : a == 5 ? -1 : 0;
      int fx = 2 * x + ix + dx, fy = 2 * y + iy + dy, fz = 2 * z + iz + dz;
      if (grid_bit(D, res, fx, fy, fz)) { tag |= (uint8_t)(1 << k); break; }
    }
  }
  return tag & (uint8_t)~center;
}

/* ------------------------------------------------------------------ */
/* a5..a11 — closing                                                   */
/* ------------------------------------------------------------------ */

static int fine_radius(const int8_t *scale, int n, int x, int y, int z) {
  return clamp_radius(scale[fine_index(x, y, z, n)]);
}

/* The erosion half of the closing from the dilation D: contour S of D,
 * closing_grid_.CopyVoxelsFrom (dilation_grid_) and ErodeBySphereMipmap
 * (GMorpho.cu:7800-7803).  pyr and tag are scratch. */
static int64_t count_nonzero(const uint8_t *a, int64_t n) {
  int64_t k = 0;
#pragma omp parallel for reduction(+ : k) schedule(static)
  for (int64_t i = 0; i < n; i++) k += a[i] != 0;
  return k;
}

static void erode_from(const uint8_t *X, const int8_t *scale, int res,
                       const int *data_res, int mode, const uint8_t *D,
                       uint8_t *S, uint8_t *C, uint64_t *pyr, uint8_t *tag,
                       int64_t *erosion_list) {
  const int N = 2 * res;
  const int64_t nc = (int64_t)res * res * res;
  if (mode == 0) {
    /* TransformToContour (Grid.cu:2381-2408) */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++)
          S[(int64_t)x + (int64_t)res * y + (int64_t)res * res * z] = contour_byte(D, res, x, y, z);
    gmo_pyramid_build(S, scale, res, pyr);
    memcpy(C, D, nc); /* closing_grid_.CopyVoxelsFrom (dilation_grid_) (GMorpho.cu:7800) */
    /* ErodeBySphereTexMipmapBaseILP2 (GMorpho.cu:4349-4647): a cell with
     * D != 0 and X != 0xff is cleared when its centre 2c+1 is eroded. */
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < data_res[2]; z++)
      for (int y = 0; y < data_res[1]; y++)
        for (int x = 0; x < data_res[0]; x++) {
          int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
          if (D[c] == 0x00 || X[c] == 0xff) continue;
          if (gmo_erode_query2(pyr, res, 2 * (2 * x + 1), 2 * (2 * y + 1), 2 * (2 * z + 1))) C[c] = 0;
        }
    /* ComputeContourBase + ErodeBySphereTexMipmapPersistentWarpILP
     * (Grid.cu:1975-2071, GMorpho.cu:5041-5375): tagged cells become
     * 0xff & ~eroded, not masked by D (GMorpho.cu:5353-5360). */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++)
          tag[(int64_t)x + (int64_t)res * y + (int64_t)res * res * z] = (uint8_t)tag_base(C, res, x, y, z);
    if (erosion_list) *erosion_list = count_nonzero(tag, nc);
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++) {
          int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
          if (!tag[c]) continue;
          uint8_t eroded = 0;
          for (int k = 0; k < 8; k++) {
            int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
            if (gmo_erode_query2(pyr, res, 2 * fx + 1, 2 * fy + 1, 2 * fz + 1)) eroded |= (uint8_t)(1 << k);
          }
          C[c] = (uint8_t)(0xff & ~eroded);
        }
  } else {
    /* contour over the whole grid: voxels outside D, 6-adjacent to D */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++) {
          uint8_t b = 0;
          int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
          for (int k = 0; k < 8; k++) {
            int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
            if ((D[c] >> k) & 1) continue;
            int adj = 0;
            if (fx > 0 && grid_bit(D, res, fx - 1, fy, fz)) adj = 1;
            if (fx < N - 1 && grid_bit(D, res, fx + 1, fy, fz)) adj = 1;
            if (fy > 0 && grid_bit(D, res, fx, fy - 1, fz)) adj = 1;
            if (fy < N - 1 && grid_bit(D, res, fx, fy + 1, fz)) adj = 1;
            if (fz > 0 && grid_bit(D, res, fx, fy, fz - 1)) adj = 1;
            if (fz < N - 1 && grid_bit(D, res, fx, fy, fz + 1)) adj = 1;
            if (adj) b |= (uint8_t)(1 << k);
          }
          S[c] = b;
        }
    gmo_pyramid_build(S, scale, res, pyr);
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++) {
          int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
          uint8_t b = D[c];
          for (int k = 0; k < 8; k++) {
            if (!((b >> k) & 1)) continue;
            int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
            if (gmo_erode_query2(pyr, res, 2 * fx + 1, 2 * fy + 1, 2 * fz + 1)) b &= (uint8_t)~(1 << k);
          }
          C[c] = b;
        }
  }
}

int gmo_close_lists(const uint8_t *X, const int8_t *scale, int res,
                    const int *data_res, int mode, int se, uint8_t *Dout,
                    uint8_t *Sout, uint8_t *Cout, int64_t *lists) {
  const int N = 2 * res;
  const int64_t nc = (int64_t)res * res * res;
  const int64_t npyr = gmo_pyramid_size(res);
  uint64_t *pyr = (uint64_t *)malloc(sizeof(uint64_t) * npyr);
  uint8_t *D = (uint8_t *)malloc(nc), *S = (uint8_t *)malloc(nc), *C = (uint8_t *)malloc(nc);
  uint8_t *tag = (uint8_t *)malloc(nc);
  if (!pyr || !D || !S || !C || !tag) return -1;

  gmo_pyramid_build(X, scale, res, pyr);
  memcpy(D, X, nc); /* dilation_grid_.CopyVoxelsFrom (input_grid_) (GMorpho.cu:7780) */

  if (mode == 0) {
    /* DilateBy{Sphere,Cube}ByTexMipmapBase (GMorpho.cu:2828-2928, 1838-1934):
     * cells inside data_res that are not full get 0xff when their child-0
     * corner 2c satisfies the predicate with its own radius. */
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < data_res[2]; z++)
      for (int y = 0; y < data_res[1]; y++)
        for (int x = 0; x < data_res[0]; x++) {
          int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
          if (X[c] == 0xff) continue;
          int r = fine_radius(scale, N, 2 * x, 2 * y, 2 * z);
          if (gmo_dilate_query(pyr, res, se, 2 * x, 2 * y, 2 * z, r)) D[c] = 0xff;
        }
    /* ComputeContourBaseTight + DilateBy*ByTexMipmap (Grid.cu:2073-2168,
     * GMorpho.cu:2930-3056): tagged cells are overwritten by the per-voxel
     * predicate of their eight fine voxels. */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++)
          tag[(int64_t)x + (int64_t)res * y + (int64_t)res * res * z] = (uint8_t)tag_tight(D, res, x, y, z);
    if (lists) lists[0] = count_nonzero(tag, nc);
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++) {
          int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
          if (!tag[c]) continue;
          uint8_t b = 0;
          for (int k = 0; k < 8; k++) {
            int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
            if (gmo_dilate_query(pyr, res, se, fx, fy, fz, fine_radius(scale, N, fx, fy, fz)))
              b |= (uint8_t)(1 << k);
          }
          D[c] = b;
        }
  } else {
    /* GM_EXACT: the reference's fine predicates at every fine voxel. */
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++) {
          uint8_t b = 0;
          for (int k = 0; k < 8; k++) {
            int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
            if (gmo_dilate_query(pyr, res, se, fx, fy, fz, fine_radius(scale, N, fx, fy, fz)))
              b |= (uint8_t)(1 << k);
          }
          D[(int64_t)x + (int64_t)res * y + (int64_t)res * res * z] = b;
        }
  }
  erode_from(X, scale, res, data_res, mode, D, S, C, pyr, tag, lists ? &lists[1] : NULL);
  if (Dout) memcpy(Dout, D, nc);
  if (Sout) memcpy(Sout, S, nc);
  if (Cout) memcpy(Cout, C, nc);
  free(pyr); free(D); free(S); free(C); free(tag);
  return 0;
}

int gmo_close(const uint8_t *X, const int8_t *scale, int res,
              const int *data_res, int mode, int se, uint8_t *Dout,
              uint8_t *Sout, uint8_t *Cout) {
  return gmo_close_lists(X, scale, res, data_res, mode, se, Dout, Sout, Cout, NULL);
}

int gmo_close_exact_brute(const uint8_t *X, const int8_t *scale, int res, int se,
                          uint8_t *Cout) {
  const int N = 2 * res;
  const int64_t nc = (int64_t)res * res * res;
  uint8_t *D = (uint8_t *)calloc(nc, 1), *S = (uint8_t *)calloc(nc, 1);
  if (!D || !S) return -1;
#pragma omp parallel for schedule(dynamic, 1)
  for (int fz = 0; fz < N; fz++)
    for (int fy = 0; fy < N; fy++)
      for (int fx = 0; fx < N; fx++) {
        if (gmo_dilate_query_brute(X, scale, res, se, fx, fy, fz, fine_radius(scale, N, fx, fy, fz))) {
          int64_t c = (int64_t)(fx >> 1) + (int64_t)res * (fy >> 1) + (int64_t)res * res * (fz >> 1);
#pragma omp atomic
          D[c] |= (uint8_t)(1 << ((fx & 1) | ((fy & 1) << 1) | ((fz & 1) << 2)));
        }
      }
  for (int fz = 0; fz < N; fz++)
    for (int fy = 0; fy < N; fy++)
      for (int fx = 0; fx < N; fx++) {
        if (grid_bit(D, res, fx, fy, fz)) continue;
        int adj = (fx > 0 && grid_bit(D, res, fx - 1, fy, fz)) || (fx < N - 1 && grid_bit(D, res, fx + 1, fy, fz)) ||
                  (fy > 0 && grid_bit(D, res, fx, fy - 1, fz)) || (fy < N - 1 && grid_bit(D, res, fx, fy + 1, fz)) ||
                  (fz > 0 && grid_bit(D, res, fx, fy, fz - 1)) || (fz < N - 1 && grid_bit(D, res, fx, fy, fz + 1));
        if (adj) {
          int64_t c = (int64_t)(fx >> 1) + (int64_t)res * (fy >> 1) + (int64_t)res * res * (fz >> 1);
          S[c] |= (uint8_t)(1 << ((fx & 1) | ((fy & 1) << 1) | ((fz & 1) << 2)));
        }
      }
  memset(Cout, 0, nc);
#pragma omp parallel for schedule(dynamic, 1)
  for (int fz = 0; fz < N; fz++)
    for (int fy = 0; fy < N; fy++)
      for (int fx = 0; fx < N; fx++) {
        if (!grid_bit(D, res, fx, fy, fz)) continue;
        if (gmo_erode_query2_brute(S, scale, res, 2 * fx + 1, 2 * fy + 1, 2 * fz + 1)) continue;
        int64_t c = (int64_t)(fx >> 1) + (int64_t)res * (fy >> 1) + (int64_t)res * res * (fz >> 1);
#pragma omp atomic
        Cout[c] |= (uint8_t)(1 << ((fx & 1) | ((fy & 1) << 1) | ((fz & 1) << 2)));
      }
  free(D); free(S);
  return 0;
}

/* ------------------------------------------------------------------ */
/* f2 — rotated-cube dilation under a quaternion field                 */
/* ------------------------------------------------------------------ */
/* The float expressions are evaluated as the reference writes them
 * (left-to-right sums; this file is compiled with -ffp-contract=off, so
 * no multiply-add is fused); the CUDA kernels evaluate the same operations
 * with explicit rounding and give the same booleans. */

typedef struct { float x, y, z, w; } quat_t;

/* Field node i.  On its top faces the reference reads one node past the
 * field (InterpolateQuaternionField, GMorpho.cu:1658-1667: x wraps to the
 * next row, y to the next slice, z past the allocation); reads past the
 * last node are clamped to it here. */
static quat_t q_node(const float *Q, int64_t n, int64_t i) {
  if (i > n - 1) i = n - 1;
  quat_t q = {Q[4 * i], Q[4 * i + 1], Q[4 * i + 2], Q[4 * i + 3]};
  return q;
}

/* (1 - t) a + t b: interpolate_cube_group with an empty group
 * (cuda_math.h:424-430, called with group size 0 at GMorpho.cu:1733, 2515) */
static quat_t q_lerp(quat_t a, quat_t b, float t) {
  const float s = 1.f - t;
  quat_t r = {s * a.x + t * b.x, s * a.y + t * b.y, s * a.z + t * b.z, s * a.w + t * b.w};
  return r;
}

/* Hamilton product a b, terms in the order of cuda_math.h:386-393 */
static quat_t q_mul(quat_t a, quat_t b) {
  quat_t r;
  r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
  r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
  r.y = a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x;
  r.z = a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w;
  return r;
}

/* InterpolateQuaternionField (GMorpho.cu:1631-1710) at lattice point
 * (ix, iy, iz) of a grid of `res` points per axis, then
 * quat = normalize (conj (quat)) and the rotated axes rotate (quat, e_k) =
 * conj(quat) (e_k, 0) quat (GMorpho.cu:1735-1745, 2517-2527;
 * cuda_math.h:396-401).  axes = b_x, b_y, b_z. */
void gmo_rotcube_frame(const float *Q, int qres, int ix, int iy, int iz, int res, float *axes) {
  const float fx = (float)qres * ((float)ix / (float)res);
  const float fy = (float)qres * ((float)iy / (float)res);
  const float fz = (float)qres * ((float)iz / (float)res);
  const int jx = (int)fx, jy = (int)fy, jz = (int)fz;
  const int64_t sy = qres, sz = (int64_t)qres * qres, n = sz * qres;
  const int64_t b = jx + sy * jy + sz * jz;
  const float tx = fx - (float)jx, ty = fy - (float)jy, tz = fz - (float)jz;
  const quat_t q00 = q_lerp(q_node(Q, n, b), q_node(Q, n, b + 1), tx);
  const quat_t q01 = q_lerp(q_node(Q, n, b + sz), q_node(Q, n, b + 1 + sz), tx);
  const quat_t q10 = q_lerp(q_node(Q, n, b + sy), q_node(Q, n, b + 1 + sy), tx);
  const quat_t q11 = q_lerp(q_node(Q, n, b + sy + sz), q_node(Q, n, b + 1 + sy + sz), tx);
  quat_t q = q_lerp(q_lerp(q00, q10, ty), q_lerp(q01, q11, ty), tz);
  q.x = -q.x;
  q.y = -q.y;
  q.z = -q.z;
  const float len = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  q.x = q.x / len;
  q.y = q.y / len;
  q.z = q.z / len;
  q.w = q.w / len;
  const quat_t qc = {-q.x, -q.y, -q.z, q.w};
  for (int a = 0; a < 3; a++) {
    const quat_t u = {a == 0 ? 1.f : 0.f, a == 1 ? 1.f : 0.f, a == 2 ? 1.f : 0.f, 0.f};
    const quat_t r = q_mul(qc, q_mul(u, q));
    axes[3 * a] = r.x;
    axes[3 * a + 1] = r.y;
    axes[3 * a + 2] = r.z;
  }
}

typedef struct {
  float c[3];            /* structuring element centre, fine units */
  float bx[3], by[3], bz[3];
  float se;              /* half size (the radius) */
} rc_query_t;

/* HasRotCubeSEOverlap (GMorpho.cu:241-302, 334-349): separating-axis test
 * of the rotated cube against the node box of centre n and half size hs,
 * t = centre - n; false as soon as one of the 15 axes separates. */
static int rc_overlap(const rc_query_t *q, float nx, float ny, float nz, float hs) {
  const float tx = q->c[0] - nx, ty = q->c[1] - ny, tz = q->c[2] - nz;
  const float *bx = q->bx, *by = q->by, *bz = q->bz;
  const float se = q->se;
  if (fabsf(tx) > hs + se * (fabsf(bx[0]) + fabsf(by[0]) + fabsf(bz[0]))) return 0;
  if (fabsf(ty) > hs + se * (fabsf(bx[1]) + fabsf(by[1]) + fabsf(bz[1]))) return 0;
  if (fabsf(tz) > hs + se * (fabsf(bx[2]) + fabsf(by[2]) + fabsf(bz[2]))) return 0;
  if (fabsf(tx * bx[0] + ty * bx[1] + tz * bx[2]) > hs * (fabsf(bx[0]) + fabsf(bx[1]) + fabsf(bx[2])) + se) return 0;
  if (fabsf(tx * by[0] + ty * by[1] + tz * by[2]) > hs * (fabsf(by[0]) + fabsf(by[1]) + fabsf(by[2])) + se) return 0;
  if (fabsf(tx * bz[0] + ty * bz[1] + tz * bz[2]) > hs * (fabsf(bz[0]) + fabsf(bz[1]) + fabsf(bz[2])) + se) return 0;
  if (fabsf(tz * bx[1] - ty * bx[2]) > hs * (fabsf(bx[2]) + fabsf(bx[1])) + se * (fabsf(bz[0]) + fabsf(by[0]))) return 0;
  if (fabsf(tz * by[1] - ty * by[2]) > hs * (fabsf(by[2]) + fabsf(by[1])) + se * (fabsf(bz[0]) + fabsf(bx[0]))) return 0;
  if (fabsf(tz * bz[1] - ty * bz[2]) > hs * (fabsf(bz[2]) + fabsf(bz[1])) + se * (fabsf(by[0]) + fabsf(bx[0]))) return 0;
  if (fabsf(tx * bx[2] - tz * bx[0]) > hs * (fabsf(bx[2]) + fabsf(bx[0])) + se * (fabsf(bz[1]) + fabsf(by[1]))) return 0;
  if (fabsf(tx * by[2] - tz * by[0]) > hs * (fabsf(by[2]) + fabsf(by[0])) + se * (fabsf(bz[1]) + fabsf(bx[1]))) return 0;
  if (fabsf(tx * bz[2] - tz * bz[0]) > hs * (fabsf(bz[2]) + fabsf(bz[0])) + se * (fabsf(by[1]) + fabsf(bx[1]))) return 0;
  if (fabsf(ty * bx[0] - tx * bx[1]) > hs * (fabsf(bx[1]) + fabsf(bx[0])) + se * (fabsf(bz[2]) + fabsf(by[2]))) return 0;
  if (fabsf(ty * by[0] - tx * by[1]) > hs * (fabsf(by[1]) + fabsf(by[0])) + se * (fabsf(bz[2]) + fabsf(bx[2]))) return 0;
  if (fabsf(ty * bz[0] - tx * bz[1]) > hs * (fabsf(bz[1]) + fabsf(bz[0])) + se * (fabsf(by[2]) + fabsf(bx[2]))) return 0;
  return 1;
}

/* Traversal of DilateByRotCubeByTexMipmap{Base,} (GMorpho.cu:1747-1831,
 * 2529-2583): true iff some occupied fine voxel is reached through nodes
 * that all overlap the rotated cube. */
static int rc_run(const uint64_t *pyr, int res, const rc_query_t *q) {
  const int L = ilog2i(res), maxd = L + 1, max_res = 1 << maxd;
  node_t stack[8 * 24];
  int sp = 0;
  stack[sp++] = (node_t){0, 0, 0, 0};
  while (sp > 0) {
    const node_t nd = stack[--sp];
    const int level = L - nd.d, nl = res >> level;
    const uint64_t tex = pyr[level_offset(res, level) + (int64_t)nd.x + (int64_t)nl * nd.y +
                             (int64_t)nl * nl * nd.z];
    const int occ = (int)(tex >> 56);
    const float ncs = (float)(max_res >> (nd.d + 1));
    for (int k = 0; k < 8; k++) {
      if (!(occ & (1 << k))) continue;
      const int bx = 2 * nd.x + (k & 1), by = 2 * nd.y + ((k >> 1) & 1), bz = 2 * nd.z + (k >> 2);
      if (!rc_overlap(q, ncs * ((float)bx + 0.5f), ncs * ((float)by + 0.5f), ncs * ((float)bz + 0.5f), 0.5f * ncs))
        continue;
      if (nd.d + 1 == maxd) return 1;
      stack[sp++] = (node_t){nd.d + 1, bx, by, bz};
    }
  }
  return 0;
}

int gmo_rotcube_query(const uint64_t *pyr, int res, const float *Q, int qres, int px, int py, int pz,
                      int frame_res, int cx, int cy, int cz, int radius) {
  rc_query_t q;
  float ax[9];
  gmo_rotcube_frame(Q, qres, px, py, pz, frame_res, ax);
  for (int i = 0; i < 3; i++) {
    q.bx[i] = ax[i];
    q.by[i] = ax[3 + i];
    q.bz[i] = ax[6 + i];
  }
  q.c[0] = (float)cx;
  q.c[1] = (float)cy;
  q.c[2] = (float)cz;
  q.se = (float)radius;
  return rc_run(pyr, res, &q);
}

/* TagVoxelsContourBaseConservative (GMorpho/Grid.cu:1464-1498): c in
 * [1, res-2]^3 whose byte differs from one of its eight diagonal
 * neighbours c + (+-1, +-1, +-1) (the loop keeps only offsets with all
 * three components non-zero). */
static int tag_conservative(const uint8_t *g, int res, int x, int y, int z) {
  if (x < 1 || y < 1 || z < 1 || x > res - 2 || y > res - 2 || z > res - 2) return 0;
  const int64_t s1 = res, s2 = (int64_t)res * res;
  const int64_t c = x + s1 * y + s2 * z;
  for (int k = 0; k < 8; k++) {
    const int64_t o = ((k & 1) ? 1 : -1) + s1 * (((k >> 1) & 1) ? 1 : -1) + s2 * ((k >> 2) ? 1 : -1);
    if (g[c + o] != g[c]) return 1;
  }
  return 0;
}

/* the eight fine voxels of cell (x, y, z), each with its own frame
 * (frame grid 2 res) and radius (GMorpho.cu:2492-2527) */
static uint8_t rc_cell_fine(const uint64_t *pyr, int res, const float *Q, int qres, int x, int y, int z) {
  const uint64_t tex = pyr[(int64_t)x + (int64_t)res * y + (int64_t)res * res * z];
  uint8_t b = 0;
  for (int k = 0; k < 8; k++) {
    const int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
    const int r = (int)((tex >> (7 * k)) & 0x7f);
    if (gmo_rotcube_query(pyr, res, Q, qres, fx, fy, fz, 2 * res, fx, fy, fz, r)) b |= (uint8_t)(1 << k);
  }
  return b;
}

int gmo_close_rotcube(const uint8_t *X, const int8_t *scale, int res, const int *data_res, const float *Q, int qres,
                      int mode, uint8_t *Dout, uint8_t *Sout, uint8_t *Cout) {
  const int64_t nc = (int64_t)res * res * res;
  uint64_t *pyr = (uint64_t *)malloc(sizeof(uint64_t) * gmo_pyramid_size(res));
  uint8_t *D = (uint8_t *)malloc(nc), *S = (uint8_t *)malloc(nc), *C = (uint8_t *)malloc(nc);
  uint8_t *tag = (uint8_t *)malloc(nc);
  if (!pyr || !D || !S || !C || !tag) return -1;
  gmo_pyramid_build(X, scale, res, pyr);
  memcpy(D, X, nc);
  if (mode == 0) {
    /* DilateByRotCubeByTexMipmapBase (GMorpho.cu:1712-1837): cells inside
     * data_res that are not full, frame at the cell (frame grid res),
     * centre 2c, radius of child 0 */
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < data_res[2]; z++)
      for (int y = 0; y < data_res[1]; y++)
        for (int x = 0; x < data_res[0]; x++) {
          const int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
          if (X[c] == 0xff) continue;
          const int r = (int)(pyr[c] & 0x7f);
          if (gmo_rotcube_query(pyr, res, Q, qres, x, y, z, res, 2 * x, 2 * y, 2 * z, r)) D[c] = 0xff;
        }
    /* ComputeContourBaseConservative + DilateByRotCubeByTexMipmap
     * (GMorpho.cu:3183-3224, 2464-2602): tagged cells are overwritten */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++)
          tag[(int64_t)x + (int64_t)res * y + (int64_t)res * res * z] = (uint8_t)tag_conservative(D, res, x, y, z);
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++) {
          const int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
          if (tag[c]) D[c] = rc_cell_fine(pyr, res, Q, qres, x, y, z);
        }
  } else {
    /* GM_EXACT: the fine predicate at every fine voxel */
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < res; z++)
      for (int y = 0; y < res; y++)
        for (int x = 0; x < res; x++)
          D[(int64_t)x + (int64_t)res * y + (int64_t)res * res * z] = rc_cell_fine(pyr, res, Q, qres, x, y, z);
  }
  erode_from(X, scale, res, data_res, mode, D, S, C, pyr, tag, NULL);
  if (Dout) memcpy(Dout, D, nc);
  if (Sout) memcpy(Sout, S, nc);
  if (Cout) memcpy(Cout, C, nc);
  free(pyr); free(D); free(S); free(C); free(tag);
  return 0;
}

/* ------------------------------------------------------------------ */
/* a12..a15 — contour marching cubes                                   */
/* ------------------------------------------------------------------ */

static const uint64_t kTriPacked[256] = GM_MC_TRI_PACKED_INIT;
static const uint8_t kTriCount[256] = GM_MC_TRI_COUNT_INIT;
static const uint8_t kTriLen[256] = GM_MC_TRI_LEN_INIT;

/* MC corner j of a cube (v0..v7 = 000,100,110,010,001,101,111,011), the
 * corner order of GMorpho.cu:6146-6232. */
static const int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                 {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

static int edge_mask(int v) {
  int m = 0;
  for (int e = 0; e < 12; e++)
    if (((v >> kEdge[e][0]) & 1) != ((v >> kEdge[e][1]) & 1)) m |= 1 << e;
  return m;
}

/* cube value of the MC cube whose min corner is fine voxel (fx,fy,fz) */
static int cube_value(const uint8_t *C, int res, int fx, int fy, int fz) {
  int v = 0;
  for (int j = 0; j < 8; j++)
    v |= grid_bit(C, res, fx + kCorner[j][0], fy + kCorner[j][1], fz + kCorner[j][2]) << j;
  return v;
}

/* mixed-cube mask of base cell c: bit k set when sub-cube k (min corner
 * 2c + o_k) is neither empty nor full; zero outside [1, res-2]^3
 * (TagVoxelsContourMCM, Grid.cu:1329-1462). */
static int cell_mixed_mask(const uint8_t *C, int res, int x, int y, int z, int *vals) {
  if (x < 1 || y < 1 || z < 1 || x > res - 2 || y > res - 2 || z > res - 2) return 0;
  int m = 0;
  for (int k = 0; k < 8; k++) {
    int v = cube_value(C, res, 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2));
    if (vals) vals[k] = v;
    if (v != 0 && v != 255) m |= 1 << k;
  }
  return m;
}

static inline int nv_owned(int em) { return (em & 1) + ((em >> 3) & 1) + ((em >> 8) & 1); }

int gmo_mc(const uint8_t *C, int res, const float *bbox_min, float cell_size,
           float iso, float *V, int64_t v_cap, uint32_t *T, int64_t t_cap,
           int64_t *nv_out, int64_t *nt_out) {
  const int64_t ncell = (int64_t)res * res * res;
  /* per cell (linear index): mixed mask, first compact cube id */
  uint8_t *mask = (uint8_t *)calloc(ncell, 1);
  int64_t *first = (int64_t *)malloc(sizeof(int64_t) * ncell);
  if (!mask || !first) return -2;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < res; z++)
    for (int y = 0; y < res; y++)
      for (int x = 0; x < res; x++)
        mask[(int64_t)x + (int64_t)res * y + (int64_t)res * res * z] =
            (uint8_t)cell_mixed_mask(C, res, x, y, z, NULL);
  /* compact order: cells sorted by Morton code (thrust::sort_by_key,
   * Grid.cu:1949-1956), eight sub-cubes each in child order, non-empty kept
   * (CompactMCMData, GMorpho.cu:6282-6345). */
  int64_t ncubes = 0;
  for (int64_t m = 0; m < ncell; m++) {
    uint32_t x = compact3((uint32_t)m), y = compact3((uint32_t)m >> 1), z = compact3((uint32_t)m >> 2);
    int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
    first[c] = ncubes;
    ncubes += __builtin_popcount(mask[c]);
  }
  int64_t *cpos = (int64_t *)malloc(sizeof(int64_t) * (ncubes + 1));
  uint8_t *cval = (uint8_t *)malloc(ncubes + 1);
  int64_t *voff = (int64_t *)malloc(sizeof(int64_t) * (ncubes + 1));
  int64_t *toff = (int64_t *)malloc(sizeof(int64_t) * (ncubes + 1));
  if (!cpos || !cval || !voff || !toff) return -2;
  int64_t id = 0;
  for (int64_t m = 0; m < ncell; m++) {
    uint32_t x = compact3((uint32_t)m), y = compact3((uint32_t)m >> 1), z = compact3((uint32_t)m >> 2);
    int64_t c = (int64_t)x + (int64_t)res * y + (int64_t)res * res * z;
    if (!mask[c]) continue;
    int vals[8];
    cell_mixed_mask(C, res, (int)x, (int)y, (int)z, vals);
    for (int k = 0; k < 8; k++) {
      if (!((mask[c] >> k) & 1)) continue;
      int fx = 2 * x + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
      cpos[id] = fx + ((int64_t)fy << 21) + ((int64_t)fz << 42);
      cval[id] = (uint8_t)vals[k];
      id++;
    }
  }
  /* countTrianglesAndVertices3D + exclusive scans (MarchingCubesMesher.cu:
   * 1297-1310, 1557-1563): owned edges 0, 3, 8 and the reference's
   * per-case triangle count. */
  int64_t nv = 0, nt = 0;
  for (int64_t i = 0; i < ncubes; i++) {
    voff[i] = nv;
    toff[i] = nt;
    nv += nv_owned(edge_mask(cval[i]));
    nt += kTriCount[cval[i]];
  }
  *nv_out = nv;
  *nt_out = nt;
  if (V == NULL || T == NULL) goto done;
  if (nv > v_cap || nt > t_cap) {
    free(mask); free(first); free(cpos); free(cval); free(voff); free(toff);
    return -1;
  }
  {
    const float cs = 0.5f * cell_size;
    /* compact id of the cube at fine min corner f, or -1 when absent */
#define CUBE_ID(FX, FY, FZ, OUT)                                                        \
  do {                                                                                   \
    int fx_ = (FX), fy_ = (FY), fz_ = (FZ);                                              \
    int64_t c_ = (int64_t)(fx_ >> 1) + (int64_t)res * (fy_ >> 1) + (int64_t)res * res * (fz_ >> 1); \
    int k_ = (fx_ & 1) | ((fy_ & 1) << 1) | ((fz_ & 1) << 2);                            \
    int m_ = mask[c_];                                                                   \
    (OUT) = ((m_ >> k_) & 1) ? first[c_] + __builtin_popcount(m_ & ((1 << k_) - 1)) : -1; \
  } while (0)
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < ncubes; i++) {
      const int fx = (int)(cpos[i] & 0x1fffff), fy = (int)((cpos[i] >> 21) & 0x1fffff),
                fz = (int)(cpos[i] >> 42);
      const int val = cval[i];
      const int em = edge_mask(val);
      /* createTrianglesAndVertices3D (MarchingCubesMesher.cu:1312-1500) */
      float px = fmaf((float)fx, cs, bbox_min[0]);
      float py = fmaf((float)fy, cs, bbox_min[1]);
      float pz = fmaf((float)fz, cs, bbox_min[2]);
      float v[8];
      for (int j = 0; j < 8; j++) v[j] = ((val >> j) & 1) ? 1.f : 0.f;
      uint32_t vert[12];
      memset(vert, 0, sizeof(vert));
      int64_t base = voff[i];
      int ind = 0;
      if (em & 1) { /* edge 0: p1 = point, p2 = point + (cs,0,0) */
        vert[0] = (uint32_t)(base + ind);
        float p2x = px + cs;
        float t = iso - v[0];
        float q = (t * (p2x - px)) / (v[1] - v[0]);
        float *o = V + 3 * (base + ind);
        o[0] = px + q;
        o[1] = py + (t * (py - py)) / (v[1] - v[0]);
        o[2] = pz + (t * (pz - pz)) / (v[1] - v[0]);
        ind++;
      }
      if (em & 8) { /* edge 3: p1 = point + (0,cs,0) (v3), p2 = point (v0) */
        vert[3] = (uint32_t)(base + ind);
        float p1y = py + cs;
        float t = iso - v[3];
        float *o = V + 3 * (base + ind);
        o[0] = px + (t * (px - px)) / (v[0] - v[3]);
        o[1] = p1y + (t * (py - p1y)) / (v[0] - v[3]);
        o[2] = pz + (t * (pz - pz)) / (v[0] - v[3]);
        ind++;
      }
      if (em & 256) { /* edge 8: p1 = point (v0), p2 = point + (0,0,cs) (v4) */
        vert[8] = (uint32_t)(base + ind);
        float p2z = pz + cs;
        float t = iso - v[0];
        float *o = V + 3 * (base + ind);
        o[0] = px + (t * (px - px)) / (v[4] - v[0]);
        o[1] = py + (t * (py - py)) / (v[4] - v[0]);
        o[2] = pz + (t * (p2z - pz)) / (v[4] - v[0]);
        ind++;
      }
      int64_t id1, id2, id3, id4, id5, id7;
      CUBE_ID(fx + 1, fy, fz, id1);
      CUBE_ID(fx + 1, fy + 1, fz, id2);
      CUBE_ID(fx, fy + 1, fz, id3);
      CUBE_ID(fx, fy, fz + 1, id4);
      CUBE_ID(fx + 1, fy, fz + 1, id5);
      CUBE_ID(fx, fy + 1, fz + 1, id7);
#define E0(ID) (edge_mask(cval[ID]) & 1)
#define E3(ID) ((edge_mask(cval[ID]) >> 3) & 1)
      if ((em & 2) && id1 >= 0) vert[1] = (uint32_t)(voff[id1] + E0(id1));
      if (em & 4) vert[2] = id3 >= 0 ? (uint32_t)voff[id3] : 0;
      if (em & 16) vert[4] = id4 >= 0 ? (uint32_t)voff[id4] : 0;
      if ((em & 32) && id5 >= 0) vert[5] = (uint32_t)(voff[id5] + E0(id5));
      if (em & 64) vert[6] = id7 >= 0 ? (uint32_t)voff[id7] : 0;
      if ((em & 128) && id4 >= 0) vert[7] = (uint32_t)(voff[id4] + E0(id4));
      if (em & 512) vert[9] = id1 >= 0 ? (uint32_t)(voff[id1] + E0(id1) + E3(id1)) : 0;
      if (em & 1024) vert[10] = id2 >= 0 ? (uint32_t)(voff[id2] + E0(id2) + E3(id2)) : 0;
      if (em & 2048) vert[11] = id3 >= 0 ? (uint32_t)(voff[id3] + E0(id3) + E3(id3)) : 0;
#undef E0
#undef E3
      /* triangles with reversed winding (MarchingCubesMesher.cu:1487-1497);
       * slot count from the reference table, so the fifth triangle of a
       * case-91 cube lands on the next cube's first slot (written below,
       * after every regular triangle) or past the end (dropped). */
      const uint64_t tl = kTriPacked[val];
      const int len = kTriCount[val] < kTriLen[val] ? kTriCount[val] : kTriLen[val];
      for (int t = 0; t < len; t++) {
        uint32_t *o = T + 3 * (toff[i] + t);
        o[0] = vert[(tl >> (4 * (3 * t + 2))) & 0xf];
        o[1] = vert[(tl >> (4 * (3 * t + 1))) & 0xf];
        o[2] = vert[(tl >> (4 * (3 * t))) & 0xf];
      }
    }
    /* case-91 extra triangles (written last: the later store wins) */
    for (int64_t i = 0; i < ncubes; i++) {
      const int val = cval[i];
      if (kTriLen[val] <= kTriCount[val]) continue;
      const int64_t slot = toff[i] + kTriCount[val];
      if (slot >= nt) continue;
      /* recompute vert[] for this cube */
      const int fx = (int)(cpos[i] & 0x1fffff), fy = (int)((cpos[i] >> 21) & 0x1fffff),
                fz = (int)(cpos[i] >> 42);
      const int em = edge_mask(val);
      uint32_t vert[12];
      memset(vert, 0, sizeof(vert));
      int64_t base = voff[i];
      int ind = 0;
      if (em & 1) vert[0] = (uint32_t)(base + ind++);
      if (em & 8) vert[3] = (uint32_t)(base + ind++);
      if (em & 256) vert[8] = (uint32_t)(base + ind++);
      int64_t id1, id2, id3, id4, id5, id7;
      CUBE_ID(fx + 1, fy, fz, id1);
      CUBE_ID(fx + 1, fy + 1, fz, id2);
      CUBE_ID(fx, fy + 1, fz, id3);
      CUBE_ID(fx, fy, fz + 1, id4);
      CUBE_ID(fx + 1, fy, fz + 1, id5);
      CUBE_ID(fx, fy + 1, fz + 1, id7);
#define E0(ID) (edge_mask(cval[ID]) & 1)
#define E3(ID) ((edge_mask(cval[ID]) >> 3) & 1)
      if ((em & 2) && id1 >= 0) vert[1] = (uint32_t)(voff[id1] + E0(id1));
      if (em & 4) vert[2] = id3 >= 0 ? (uint32_t)voff[id3] : 0;
      if (em & 16) vert[4] = id4 >= 0 ? (uint32_t)voff[id4] : 0;
      if ((em & 32) && id5 >= 0) vert[5] = (uint32_t)(voff[id5] + E0(id5));
      if (em & 64) vert[6] = id7 >= 0 ? (uint32_t)voff[id7] : 0;
      if ((em & 128) && id4 >= 0) vert[7] = (uint32_t)(voff[id4] + E0(id4));
      if (em & 512) vert[9] = id1 >= 0 ? (uint32_t)(voff[id1] + E0(id1) + E3(id1)) : 0;
      if (em & 1024) vert[10] = id2 >= 0 ? (uint32_t)(voff[id2] + E0(id2) + E3(id2)) : 0;
      if (em & 2048) vert[11] = id3 >= 0 ? (uint32_t)(voff[id3] + E0(id3) + E3(id3)) : 0;
#undef E0
#undef E3
      const uint64_t tl = kTriPacked[val];
      const int t = kTriCount[val];
      uint32_t *o = T + 3 * slot;
      o[0] = vert[(tl >> (4 * (3 * t + 2))) & 0xf];
      o[1] = vert[(tl >> (4 * (3 * t + 1))) & 0xf];
      o[2] = vert[(tl >> (4 * (3 * t))) & 0xf];
    }
#undef CUBE_ID
  }
done:
  free(mask); free(first); free(cpos); free(cval); free(voff); free(toff);
  return 0;
}

/* ------------------------------------------------------------------ */
/* a16 — normals and bilateral normal filtering                        */
/* ------------------------------------------------------------------ */

static void normalize3(float *n) {
  float l = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  n[0] = n[0] / l;
  n[1] = n[1] / l;
  n[2] = n[2] / l;
}

static float dist2(const float *a, const float *b) {
  float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  return dx * dx + dy * dy + dz * dz;
}

void gmo_normals(const float *V, int64_t nv, const uint32_t *T, int64_t nt,
                 int iters, float *N) {
  /* ComputeMeshNormals + NormalizeMeshNormals (GMorpho.cu:6498-6537) */
  memset(N, 0, sizeof(float) * 3 * nv);
  for (int64_t t = 0; t < nt; t++) {
    const float *p0 = V + 3 * T[3 * t], *p1 = V + 3 * T[3 * t + 1], *p2 = V + 3 * T[3 * t + 2];
    float a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    float b[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    float n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    for (int j = 0; j < 3; j++) {
      float *o = N + 3 * T[3 * t + j];
      o[0] += n[0]; o[1] += n[1]; o[2] += n[2];
    }
  }
  for (int64_t i = 0; i < nv; i++) normalize3(N + 3 * i);
  /* BilateralMeshFiltering{,Normalize} (GMorpho.cu:6539-6620), sigmas of
   * GMorpho.cu:6959-6969 */
  float *B = (float *)malloc(sizeof(float) * 3 * (nv > 0 ? nv : 1));
  for (int it = 0; it < iters; it++) {
    const float sp = 1.f, sn = it < 2 ? 1e10f : 0.2f;
    const float sp2 = sp * sp, sn2 = sn * sn;
    memset(B, 0, sizeof(float) * 3 * nv);
    for (int64_t t = 0; t < nt; t++) {
      const uint32_t id[3] = {T[3 * t], T[3 * t + 1], T[3 * t + 2]};
      for (int a = 0; a < 3; a++) {
        const int b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
        const float *pa = V + 3 * id[a], *pb = V + 3 * id[b], *pc = V + 3 * id[c];
        const float *na = N + 3 * id[a], *nb = N + 3 * id[b], *nc = N + 3 * id[c];
        float w1 = expf(-(dist2(pa, pb) / sp2 + dist2(na, nb) / sn2));
        float w2 = expf(-(dist2(pa, pc) / sp2 + dist2(na, nc) / sn2));
        float *o = B + 3 * id[a];
        o[0] += w1 * nb[0] + w2 * nc[0];
        o[1] += w1 * nb[1] + w2 * nc[1];
        o[2] += w1 * nb[2] + w2 * nc[2];
      }
    }
    for (int64_t i = 0; i < nv; i++) {
      normalize3(B + 3 * i);
      N[3 * i] = B[3 * i]; N[3 * i + 1] = B[3 * i + 1]; N[3 * i + 2] = B[3 * i + 2];
    }
  }
  free(B);
}

/* ------------------------------------------------------------------ */
/* a3 — ScaleField brush                                               */
/* ------------------------------------------------------------------ */

/* UpdateScaleGrid (GMorpho/ScaleField.cu:81-141) with tukey
 * (GMorpho/cuda_math.h:696-704).  The float operations are spelled out in a
 * fixed order so that the CUDA kernel can reproduce them exactly. */
void gmo_scale_brush(int8_t *scale, int n, const float *bbox_min,
                     float cell_size, const float *pos, float sv,
                     float support, float global_scale, int mode) {
  const float v = sv;
  const float h = (support - v) / sqrtf(1.f - sqrtf(0.5f));
#pragma omp parallel for schedule(static)
  for (int z = 0; z < n; z++)
    for (int y = 0; y < n; y++)
      for (int x = 0; x < n; x++) {
        float ux = fmaf(cell_size, (float)x, bbox_min[0]) - pos[0];
        float uy = fmaf(cell_size, (float)y, bbox_min[1]) - pos[1];
        float uz = fmaf(cell_size, (float)z, bbox_min[2]) - pos[2];
        float d = sqrtf(fmaf(uz, uz, fmaf(uy, uy, ux * ux)));
        if (!(d < v + h)) continue;
        float w;
        if (d < v) w = 1.f;
        else {
          float a = (d - v) / h;
          float b = 1.f - a * a;
          w = b * b;
        }
        int64_t i = fine_index(x, y, z, n);
        float prev = (float)scale[i];
        float target = mode == 3 ? global_scale / cell_size : sv / cell_size;
        float dist = prev * (1.f - w) + w * target;
        dist = floorf(dist);
        dist = fmaxf(fminf(dist, 127.f), 0.f);
        if (mode == 1) scale[i] = (int8_t)floorf(fmaxf(dist, prev));
        else if (mode == 2) scale[i] = (int8_t)floorf(fminf(dist, prev));
        else if (mode == 3) scale[i] = (int8_t)dist;
      }
}

/* ------------------------------------------------------------------ */
/* a2 — voxelizer                                                      */
/* ------------------------------------------------------------------ */

void gmo_grid_attributes(const float *P, int64_t nv, int base_res, float margin,
                         float *bmin, float *bmax, float *cell, int *data_res) {
  /* Voxelizer::ComputeGridAttributes (GMorpho/Voxelizer.cu:431-455) */
  float mn[3] = {P[0], P[1], P[2]}, mx[3] = {P[0], P[1], P[2]};
  for (int64_t i = 0; i < nv; i++)
    for (int a = 0; a < 3; a++) {
      float v = P[3 * i + a];
      if (v < mn[a]) mn[a] = v;
      if (v > mx[a]) mx[a] = v;
    }
  float ext = fmaxf(fabsf(mx[0] - mn[0]), fmaxf(fabsf(mx[1] - mn[1]), fabsf(mx[2] - mn[2])));
  float thickness = ext / (float)base_res;
  float off = 2.f * thickness + margin;
  for (int a = 0; a < 3; a++) {
    mn[a] -= off;
    mx[a] += off;
  }
  float c = fmaxf(fabsf(mx[0] - mn[0]), fmaxf(fabsf(mx[1] - mn[1]), fabsf(mx[2] - mn[2]))) / (float)base_res;
  for (int a = 0; a < 3; a++) {
    bmin[a] = mn[a];
    bmax[a] = mx[a];
    data_res[a] = (int)ceilf((mx[a] - mn[a]) / c);
  }
  *cell = c;
}

/* Triangle / closed-box overlap by the separating-axis theorem (13 axes). */
static int tri_box_overlap(const double c[3], double half, const double v0[3],
                           const double v1[3], const double v2[3]) {
  double a[3], b[3], d[3];
  for (int i = 0; i < 3; i++) {
    a[i] = v0[i] - c[i];
    b[i] = v1[i] - c[i];
    d[i] = v2[i] - c[i];
  }
  const double *vv[3] = {a, b, d};
  for (int ax = 0; ax < 3; ax++) {
    double mn = a[ax], mx = a[ax];
    if (b[ax] < mn) mn = b[ax];
    if (b[ax] > mx) mx = b[ax];
    if (d[ax] < mn) mn = d[ax];
    if (d[ax] > mx) mx = d[ax];
    if (mn > half || mx < -half) return 0;
  }
  double e[3][3];
  for (int i = 0; i < 3; i++) {
    e[0][i] = b[i] - a[i];
    e[1][i] = d[i] - b[i];
    e[2][i] = a[i] - d[i];
  }
  double nrm[3] = {e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
                   e[0][0] * e[1][1] - e[0][1] * e[1][0]};
  double dd = nrm[0] * a[0] + nrm[1] * a[1] + nrm[2] * a[2];
  double rr = half * (fabs(nrm[0]) + fabs(nrm[1]) + fabs(nrm[2]));
  if (dd > rr || dd < -rr) return 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      /* axis = unit_j x e_i */
      double ax[3] = {0, 0, 0};
      if (j == 0) { ax[1] = -e[i][2]; ax[2] = e[i][1]; }
      if (j == 1) { ax[0] = e[i][2]; ax[2] = -e[i][0]; }
      if (j == 2) { ax[0] = -e[i][1]; ax[1] = e[i][0]; }
      double p0 = ax[0] * vv[0][0] + ax[1] * vv[0][1] + ax[2] * vv[0][2];
      double p1 = ax[0] * vv[1][0] + ax[1] * vv[1][1] + ax[2] * vv[1][2];
      double p2 = ax[0] * vv[2][0] + ax[1] * vv[2][1] + ax[2] * vv[2][2];
      double mn = p0, mx = p0;
      if (p1 < mn) mn = p1;
      if (p1 > mx) mx = p1;
      if (p2 < mn) mn = p2;
      if (p2 > mx) mx = p2;
      double r = half * (fabs(ax[0]) + fabs(ax[1]) + fabs(ax[2]));
      if (mn > r || mx < -r) return 0;
    }
  return 1;
}

/* top-left coverage rule for a counter-clockwise triangle in the xy plane */
static int edge_covers(double ax, double ay, double bx, double by, double px, double py) {
  double w = (bx - ax) * (py - ay) - (by - ay) * (px - ax);
  if (w > 0) return 1;
  if (w < 0) return 0;
  /* on the edge: accept "top" (horizontal, pointing left) and "left"
   * (pointing down) edges of a CCW triangle */
  double ex = bx - ax, ey = by - ay;
  return (ey == 0 && ex < 0) || (ey < 0);
}

void gmo_voxelize(const float *P, int64_t nv, const uint32_t *T, int64_t nf,
                  int res, const float *bbox_min, float cell_size, uint8_t *grid) {
  (void)nv;
  const int N = 2 * res;
  const double h = 0.5 * (double)cell_size;
  const int64_t nvox = (int64_t)N * N * N;
  uint8_t *mark = (uint8_t *)calloc(nvox, 1);
  uint8_t *surf = (uint8_t *)calloc(nvox, 1);
  for (int64_t t = 0; t < nf; t++) {
    double g[3][3];
    for (int j = 0; j < 3; j++)
      for (int a = 0; a < 3; a++) g[j][a] = ((double)P[3 * T[3 * t + j] + a] - (double)bbox_min[a]) / h;
    /* (i) volume: pixel centres inside the xy projection flip every voxel
     * at or below the interpolated depth (vol_vox_bit.frag:35-51). */
    double area = (g[1][0] - g[0][0]) * (g[2][1] - g[0][1]) - (g[1][1] - g[0][1]) * (g[2][0] - g[0][0]);
    if (area != 0) {
      int o1 = 1, o2 = 2;
      if (area < 0) { o1 = 2; o2 = 1; area = -area; }
      const double *A = g[0], *B = g[o1], *Cc = g[o2];
      double mnx = fmin(A[0], fmin(B[0], Cc[0])), mxx = fmax(A[0], fmax(B[0], Cc[0]));
      double mny = fmin(A[1], fmin(B[1], Cc[1])), mxy = fmax(A[1], fmax(B[1], Cc[1]));
      int x0 = (int)floor(mnx - 0.5), x1 = (int)ceil(mxx - 0.5);
      int y0 = (int)floor(mny - 0.5), y1 = (int)ceil(mxy - 0.5);
      if (x0 < 0) x0 = 0;
      if (y0 < 0) y0 = 0;
      if (x1 > N - 1) x1 = N - 1;
      if (y1 > N - 1) y1 = N - 1;
      for (int y = y0; y <= y1; y++)
        for (int x = x0; x <= x1; x++) {
          double px = x + 0.5, py = y + 0.5;
          if (!edge_covers(A[0], A[1], B[0], B[1], px, py)) continue;
          if (!edge_covers(B[0], B[1], Cc[0], Cc[1], px, py)) continue;
          if (!edge_covers(Cc[0], Cc[1], A[0], A[1], px, py)) continue;
          double wa = (B[0] - px) * (Cc[1] - py) - (B[1] - py) * (Cc[0] - px);
          double wb = (Cc[0] - px) * (A[1] - py) - (Cc[1] - py) * (A[0] - px);
          double wc = area - wa - wb;
          double z = (wa * A[2] + wb * B[2] + wc * Cc[2]) / area;
          int k = (int)floor(z);
          if (k < 0) continue;
          if (k > N - 1) k = N - 1;
          mark[(int64_t)x + (int64_t)N * y + (int64_t)N * N * k] ^= 1;
        }
    }
    /* (ii) surface: voxels whose closed box meets the triangle; skinny
     * triangles (squared aspect ratio >= 50^2) are skipped as in
     * surf_vox_conserv.geo:41-70,108 and Voxelizer.cu:680. */
    double d0[3], d1[3], d2[3];
    for (int a = 0; a < 3; a++) {
      d0[a] = g[0][a] - g[1][a];
      d1[a] = g[1][a] - g[2][a];
      d2[a] = g[2][a] - g[0][a];
    }
    double l0 = d0[0] * d0[0] + d0[1] * d0[1] + d0[2] * d0[2];
    double l1 = d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2];
    double l2 = d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2];
    double maxl2 = l0 > l1 ? l0 : l1;
    if (l2 > maxl2) maxl2 = l2;
    double cx = d0[1] * d2[2] - d0[2] * d2[1], cy = d0[2] * d2[0] - d0[0] * d2[2], cz = d0[0] * d2[1] - d0[1] * d2[0];
    double a2 = cx * cx + cy * cy + cz * cz;
    if (!(a2 > 0) || !((maxl2 * maxl2) / a2 < 2500.0)) continue;
    int lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
      double mn = fmin(g[0][a], fmin(g[1][a], g[2][a])), mx = fmax(g[0][a], fmax(g[1][a], g[2][a]));
      lo[a] = (int)floor(mn) - 1;
      hi[a] = (int)floor(mx) + 1;
      if (lo[a] < 0) lo[a] = 0;
      if (hi[a] > N - 1) hi[a] = N - 1;
    }
    for (int z = lo[2]; z <= hi[2]; z++)
      for (int y = lo[1]; y <= hi[1]; y++)
        for (int x = lo[0]; x <= hi[0]; x++) {
          double c[3] = {x + 0.5, y + 0.5, z + 0.5};
          if (tri_box_overlap(c, 0.5, g[0], g[1], g[2])) surf[(int64_t)x + (int64_t)N * y + (int64_t)N * N * z] = 1;
        }
  }
  for (int y = 0; y < N; y++)
    for (int x = 0; x < N; x++) {
      int par = 0;
      for (int z = N - 1; z >= 0; z--) {
        int64_t i = (int64_t)x + (int64_t)N * y + (int64_t)N * N * z;
        par ^= mark[i];
        if (par || surf[i]) {
          int64_t c = (int64_t)(x >> 1) + (int64_t)res * (y >> 1) + (int64_t)res * res * (z >> 1);
          grid[c] |= (uint8_t)(1 << ((x & 1) | ((y & 1) << 1) | ((z & 1) << 2)));
        }
      }
    }
  free(mark);
  free(surf);
}
