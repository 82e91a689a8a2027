// framefield.cu — the frame field's biharmonic quaternion system (reference:
// FrameField::Generate with BiHarmonicSystem, GMorpho/FrameField.cu:556-575;
// FrameField::BuildSparseLTLMatrix, BuildSparseSMatrix,
// BuildSparseBiharmonicSystem, SolveSparseBiharmonicSystem,
// GMorpho/FrameFieldSparseBiharmonic.cu:170-647).
//
// System, per quaternion component k (x, y, z, w) on the res^3 lattice:
//   (L^T L + S) q_k = b_k
// L: the degree-normalised 6-neighbour Laplacian, row i = 1 on the diagonal
// and -1/deg(i) on each in-bounds neighbour (the reference builds these
// entries in float: -(1.f / deg) is used here too); S: 1 on the diagonal
// of every hard-constrained node; b_k: the constraint quaternion's
// component at those nodes.
//
// The reference factors L^T L + S with a float sparse Cholesky
// (cusolverSp).  Here the four systems are solved together, matrix-free,
// by conjugate gradients in double precision: L p and L^T y are 7-point
// stencils (no matrix is stored), the dot products are block partial sums
// reduced in a fixed order by a one-block kernel (bit-reproducible), and
// the iteration is a CUDA graph of kFfGraphIters iterations replayed until
// every component's residual is below tol * |b_k| (or zero).
#include <vector>

#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

namespace {

constexpr int kFfThreads = 256;
constexpr int kFfGraphIters = 32;

// scalar slots (doubles, 4 per name)
enum { kRR = 0, kRRNew = 4, kPAP = 8, kAlpha = 12, kBeta = 16, kBB = 20, kScalars = 24 };

__device__ __forceinline__ int ff_deg(int x, int y, int z, int n) {
  return (x > 0) + (x < n - 1) + (y > 0) + (y < n - 1) + (z > 0) + (z < n - 1);
}

// the reference's off-diagonal entry -(1.f / deg), in float, widened
__device__ __forceinline__ double ff_w(int deg) { return (double)(-(1.f / (float)deg)); }

struct V4 {
  double v[4];
};

__device__ __forceinline__ V4 ld4(const double* a, int64_t i) {
  const double2 lo = reinterpret_cast<const double2*>(a)[2 * i], hi = reinterpret_cast<const double2*>(a)[2 * i + 1];
  return V4{{lo.x, lo.y, hi.x, hi.y}};
}
__device__ __forceinline__ void st4(double* a, int64_t i, const V4& x) {
  reinterpret_cast<double2*>(a)[2 * i] = make_double2(x.v[0], x.v[1]);
  reinterpret_cast<double2*>(a)[2 * i + 1] = make_double2(x.v[2], x.v[3]);
}

// block sum of 4 doubles per thread into part[4 * blockIdx.x + k]
__device__ void ff_block_sum(const double (&s)[4], double* part) {
  __shared__ double red[kFfThreads / 32][4];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    double v = s[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0;
    for (int w = 0; w < kFfThreads / 32; w++) t += red[w][threadIdx.x];
    part[4 * blockIdx.x + threadIdx.x] = t;
  }
}

// y = L p
__global__ void __launch_bounds__(kFfThreads) k_ff_lap(const double* __restrict__ p, double* __restrict__ y, int n) {
  const int64_t total = (int64_t)n * n * n;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int x = (int)(i % n), yy = (int)((i / n) % n), z = (int)(i / ((int64_t)n * n));
  const double w = ff_w(ff_deg(x, yy, z, n));
  V4 s{{0, 0, 0, 0}};
  auto add = [&](int64_t j) {
    const V4 a = ld4(p, j);
#pragma unroll
    for (int k = 0; k < 4; k++) s.v[k] += a.v[k];
  };
  const int64_t sy = n, sz = (int64_t)n * n;
  if (z > 0) add(i - sz);
  if (yy > 0) add(i - sy);
  if (x > 0) add(i - 1);
  if (x < n - 1) add(i + 1);
  if (yy < n - 1) add(i + sy);
  if (z < n - 1) add(i + sz);
  const V4 c = ld4(p, i);
  V4 o;
#pragma unroll
  for (int k = 0; k < 4; k++) o.v[k] = c.v[k] + w * s.v[k];
  st4(y, i, o);
}

// Ap = L^T y + S p, and the block partials of p . Ap
__global__ void __launch_bounds__(kFfThreads) k_ff_lapt(const double* __restrict__ y, const double* __restrict__ p,
                                                        const uint8_t* __restrict__ S, double* __restrict__ Ap,
                                                        double* __restrict__ part, int n) {
  const int64_t total = (int64_t)n * n * n;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double dot[4] = {0, 0, 0, 0};
  if (i < total) {
    const int x = (int)(i % n), yy = (int)((i / n) % n), z = (int)(i / ((int64_t)n * n));
    V4 o = ld4(y, i);
    auto add = [&](int64_t j, int jx, int jy, int jz) {
      const double w = ff_w(ff_deg(jx, jy, jz, n));
      const V4 a = ld4(y, j);
#pragma unroll
      for (int k = 0; k < 4; k++) o.v[k] += w * a.v[k];
    };
    const int64_t sy = n, sz = (int64_t)n * n;
    if (z > 0) add(i - sz, x, yy, z - 1);
    if (yy > 0) add(i - sy, x, yy - 1, z);
    if (x > 0) add(i - 1, x - 1, yy, z);
    if (x < n - 1) add(i + 1, x + 1, yy, z);
    if (yy < n - 1) add(i + sy, x, yy + 1, z);
    if (z < n - 1) add(i + sz, x, yy, z + 1);
    const V4 pc = ld4(p, i);
    if (S[i]) {
#pragma unroll
      for (int k = 0; k < 4; k++) o.v[k] += pc.v[k];
    }
    st4(Ap, i, o);
#pragma unroll
    for (int k = 0; k < 4; k++) dot[k] = pc.v[k] * o.v[k];
  }
  ff_block_sum(dot, part);
}

// x += alpha p, r -= alpha Ap, partials of r . r
__global__ void __launch_bounds__(kFfThreads) k_ff_update(double* __restrict__ x, double* __restrict__ r,
                                                          const double* __restrict__ p, const double* __restrict__ Ap,
                                                          const double* __restrict__ sc, double* __restrict__ part,
                                                          int64_t total) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double dot[4] = {0, 0, 0, 0};
  if (i < total) {
    V4 xv = ld4(x, i), rv = ld4(r, i);
    const V4 pv = ld4(p, i), av = ld4(Ap, i);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const double a = sc[kAlpha + k];
      xv.v[k] += a * pv.v[k];
      rv.v[k] -= a * av.v[k];
      dot[k] = rv.v[k] * rv.v[k];
    }
    st4(x, i, xv);
    st4(r, i, rv);
  }
  ff_block_sum(dot, part);
}

// p = r + beta p
__global__ void __launch_bounds__(kFfThreads) k_ff_dir(double* __restrict__ p, const double* __restrict__ r,
                                                       const double* __restrict__ sc, int64_t total) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= total) return;
  V4 pv = ld4(p, i);
  const V4 rv = ld4(r, i);
#pragma unroll
  for (int k = 0; k < 4; k++) pv.v[k] = rv.v[k] + sc[kBeta + k] * pv.v[k];
  st4(p, i, pv);
}

// one block: reduce the partials of `nb` blocks in a fixed order, then
// phase 0: rr = bb = sum (start); 1: alpha = rr / pAp; 2: beta = rr' / rr, rr = rr'
__global__ void __launch_bounds__(kFfThreads) k_ff_scalars(const double* __restrict__ part, int nb,
                                                           double* __restrict__ sc, int phase) {
  __shared__ double red[kFfThreads][4];
  double s[4] = {0, 0, 0, 0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < 4; k++) s[k] += part[4 * b + k];
#pragma unroll
  for (int k = 0; k < 4; k++) red[threadIdx.x][k] = s[k];
  __syncthreads();
  for (int h = kFfThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
#pragma unroll
      for (int k = 0; k < 4; k++) red[threadIdx.x][k] += red[threadIdx.x + h][k];
    __syncthreads();
  }
  if (threadIdx.x < 4) {
    const int k = threadIdx.x;
    const double t = red[0][k];
    if (phase == 0) {
      sc[kRR + k] = t;
      sc[kBB + k] = t;
      sc[kAlpha + k] = 0;
      sc[kBeta + k] = 0;
    } else if (phase == 1) {
      sc[kPAP + k] = t;
      sc[kAlpha + k] = t > 0 ? sc[kRR + k] / t : 0.0;
    } else {
      const double rr = sc[kRR + k];
      sc[kBeta + k] = rr > 0 ? t / rr : 0.0;
      sc[kRRNew + k] = t;
      sc[kRR + k] = t;
    }
  }
}

// partials of r . r for the start
__global__ void __launch_bounds__(kFfThreads) k_ff_dot_rr(const double* __restrict__ r, double* __restrict__ part,
                                                          int64_t total) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double dot[4] = {0, 0, 0, 0};
  if (i < total) {
    const V4 rv = ld4(r, i);
#pragma unroll
    for (int k = 0; k < 4; k++) dot[k] = rv.v[k] * rv.v[k];
  }
  ff_block_sum(dot, part);
}

__global__ void k_ff_store(const double* __restrict__ x, float4* __restrict__ q, int64_t total) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const V4 v = ld4(x, i);
    q[i] = make_float4((float)v.v[0], (float)v.v[1], (float)v.v[2], (float)v.v[3]);
  }
}

__global__ void k_ff_fill(float4* __restrict__ q, float4 v, int64_t total) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    q[i] = v;
}

int ff_blocks(int64_t total) { return (int)((total + kFfThreads - 1) / kFfThreads); }

void ff_iteration(FrameFieldGpu& f, cudaStream_t st, KernelCounter* kc) {
  const int64_t total = (int64_t)f.res * f.res * f.res;
  const int nb = ff_blocks(total);
  GM_LAUNCH(kc, "k_ff_lap", st, k_ff_lap<<<nb, kFfThreads, 0, st>>>(f.p, f.y, f.res));
  GM_LAUNCH(kc, "k_ff_lapt", st, k_ff_lapt<<<nb, kFfThreads, 0, st>>>(f.y, f.p, f.S, f.Ap, f.part, f.res));
  GM_LAUNCH(kc, "k_ff_scalars", st, k_ff_scalars<<<1, kFfThreads, 0, st>>>(f.part, nb, f.sc, 1));
  GM_LAUNCH(kc, "k_ff_update", st, k_ff_update<<<nb, kFfThreads, 0, st>>>(f.x, f.r, f.p, f.Ap, f.sc, f.part, total));
  GM_LAUNCH(kc, "k_ff_scalars", st, k_ff_scalars<<<1, kFfThreads, 0, st>>>(f.part, nb, f.sc, 2));
  GM_LAUNCH(kc, "k_ff_dir", st, k_ff_dir<<<nb, kFfThreads, 0, st>>>(f.p, f.r, f.sc, total));
}

}  // namespace

cudaError_t frame_field_alloc(FrameFieldGpu& f, int res) {
  frame_field_free(f);
  const int64_t total = (int64_t)res * res * res;
  const int nb = ff_blocks(total);
  f.res = res;
  cudaError_t e;
  if ((e = cudaMalloc(&f.quats, sizeof(float4) * total)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&f.vecs, sizeof(double) * 4 * total * 5)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&f.part, sizeof(double) * 4 * nb)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&f.sc, sizeof(double) * kScalars)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&f.S, total)) != cudaSuccess) return e;
  f.x = f.vecs;
  f.r = f.x + 4 * total;
  f.p = f.r + 4 * total;
  f.y = f.p + 4 * total;
  f.Ap = f.y + 4 * total;
  if ((e = cudaMallocHost(&f.h_sc, sizeof(double) * kScalars)) != cudaSuccess) return e;
  return cudaSuccess;
}

void frame_field_free(FrameFieldGpu& f) {
  if (f.graph) cudaGraphExecDestroy(f.graph);
  cudaFree(f.quats);
  cudaFree(f.vecs);
  cudaFree(f.part);
  cudaFree(f.sc);
  cudaFree(f.S);
  if (f.h_sc) cudaFreeHost(f.h_sc);
  f = FrameFieldGpu{};
}

cudaError_t frame_field_fill(FrameFieldGpu& f, float qx, float qy, float qz, float qw, cudaStream_t st,
                             KernelCounter* kc) {
  const int64_t total = (int64_t)f.res * f.res * f.res;
  int b = ff_blocks(total);
  if (b > 152 * 8) b = 152 * 8;
  GM_LAUNCH(kc, "k_ff_fill", st, k_ff_fill<<<b, kFfThreads, 0, st>>>(f.quats, make_float4(qx, qy, qz, qw), total));
  return cudaGetLastError();
}

cudaError_t frame_field_solve(FrameFieldGpu& f, const int64_t* nodes, const float* rhs4, int npts, double tol,
                              int max_iters, int* iters_out, cudaStream_t st, KernelCounter* kc) {
  const int64_t total = (int64_t)f.res * f.res * f.res;
  const int nb = ff_blocks(total);
  cudaError_t e;
  // S and b (= r = p at x = 0): points in order, the last one on a node wins
  std::vector<double> b(4 * (size_t)npts);
  if ((e = cudaMemsetAsync(f.S, 0, total, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(f.vecs, 0, sizeof(double) * 4 * total * 5, st)) != cudaSuccess) return e;
  const uint8_t one = 1;
  for (int c = 0; c < npts; c++) {
    for (int k = 0; k < 4; k++) b[4 * c + k] = (double)rhs4[4 * c + k];
    if ((e = cudaMemcpyAsync(f.S + nodes[c], &one, 1, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(f.r + 4 * nodes[c], &b[4 * c], 4 * sizeof(double), cudaMemcpyHostToDevice, st)) !=
        cudaSuccess)
      return e;
  }
  if ((e = cudaMemcpyAsync(f.p, f.r, sizeof(double) * 4 * total, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
    return e;
  GM_LAUNCH(kc, "k_ff_dot_rr", st, k_ff_dot_rr<<<nb, kFfThreads, 0, st>>>(f.r, f.part, total));
  GM_LAUNCH(kc, "k_ff_scalars", st, k_ff_scalars<<<1, kFfThreads, 0, st>>>(f.part, nb, f.sc, 0));
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (!f.graph) {
    // kFfGraphIters iterations as one graph (the buffers never move)
    cudaStream_t cs;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) return e;
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      for (int it = 0; it < kFfGraphIters; it++) ff_iteration(f, cs, nullptr);
      e = cudaStreamEndCapture(cs, &g);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&f.graph, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return e;
  }
  int iters = 0;
  for (;;) {
    if ((e = cudaMemcpyAsync(f.h_sc, f.sc, sizeof(double) * kScalars, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    bool done = true;
    for (int k = 0; k < 4; k++) {
      const double rr = f.h_sc[kRR + k], bb = f.h_sc[kBB + k];
      if (rr > tol * tol * bb) done = false;
    }
    if (done || iters >= max_iters) break;
    if ((e = cudaGraphLaunch(f.graph, st)) != cudaSuccess) return e;
    if (kc) kc->launches += 6 * kFfGraphIters;
    iters += kFfGraphIters;
  }
  if (iters_out) *iters_out = iters;
  int bs = nb > 152 * 8 ? 152 * 8 : nb;
  GM_LAUNCH(kc, "k_ff_store", st, k_ff_store<<<bs, kFfThreads, 0, st>>>(f.x, f.quats, total));
  return cudaGetLastError();
}

}  // namespace gm
