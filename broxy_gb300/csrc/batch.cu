// batch.cu — many independent closings + meshes in one call (the batched
// form of GMorpho::Update for a set of uneven grids).
//
// Instances are spread over L "lanes" (CUDA streams, each with its own
// workspace), largest first onto the least-loaded lane, so that the small
// kernels of small grids run side by side instead of one grid at a time.
// The closing phase of a uniform-radius batch is captured once into a CUDA
// graph (fork/join over the lane streams) and replayed while the batch
// signature (pointers, sizes, radii, mode) does not change.  Meshing runs on
// the same lanes with a single host synchronisation for all the vertex and
// triangle counts.  The lane count is chosen by a small autotuner (timed
// candidates 1, 2, 4, 8, 16 on the first call of a signature).
//
// Each grid is closed on its occupied extent only: the cube at the origin
// holding every non-empty cell plus the dilation reach, rounded up to 32
// cells.  The closing is empty beyond the dilation of the input, and inside
// that cube it equals the whole grid's (no input is cut off, and the border
// rules of the last cells act on empty cells), so the result embedded back
// into the grid, and its mesh, are the whole-grid ones.  A grid of edge E
// stored in a power-of-two cube P (the reference's requirement) costs E^3
// instead of P^3.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <vector>

#include "../../include/gmorpho_gb300.h"
#include "gm_common.cuh"
#include "gm_internal.h"

namespace gm {

constexpr int kBatchGrouped = GM_BATCH_GROUPED;  // one launch per min-plus pass for all grids
constexpr int kGroupedLanes = 4;   // streams for the grouped form's per-grid kernels

struct BatchLane {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  cudaStream_t em = nullptr;       // mesh emission of the lane's grids (beside its later closings)
  cudaEvent_t em_done = nullptr;
  uint8_t* ws = nullptr;
  size_t ws_bytes = 0;
  uint8_t *Xc = nullptr, *Cc = nullptr;  // crop buffers (radius fields are read in place)
  size_t crop_cells = 0;
};

struct BatchState {
  int inject_fail = 0;  // lane buffer allocations still to fail as out of memory (fault injection)
  std::vector<BatchLane> lanes;
  std::vector<MeshBuffers> meshes;
  std::vector<int64_t> nv, nt;
  std::vector<cudaEvent_t> ev_count;  // per grid: its mesh counts are on the host
  uint32_t* h_tot = nullptr;  // pinned, 4 per instance
  int h_tot_cap = 0;
  int* d_rmax = nullptr;      // one int per instance
  int* h_rmax = nullptr;      // pinned
  int rmax_cap = 0;
  unsigned* d_ext = nullptr;  // occupied extent, 3 per instance
  unsigned* h_ext = nullptr;  // pinned
  int ext_cap = 0;
  void* d_filter = nullptr;   // table of the grouped normal filtering (mesh_filter_table_bytes)
  void* h_filter = nullptr;   // pinned
  int filter_cap = 0;
  // grouped form: per-grid workspaces (all grids' closings are in flight
  // together) and the min-plus pass of each phase, one set for live runs
  // and one owned by the captured graph
  uint8_t* arena = nullptr;
  size_t arena_bytes = 0;
  std::vector<size_t> arena_off;  // per grid: workspace, then crop buffers
  std::vector<DpxGroup*> groups[2];
  cudaEvent_t fork = nullptr;
  cudaStream_t cap_st = nullptr;  // capture / replay stream (the caller's may be the legacy stream)
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t graph = nullptr;
  uint64_t graph_sig = 0;
  long long graph_kernels = 0;
  std::map<uint64_t, int> tuned;
  int last_tuned = 0;  // the form chosen by the latest tuning
};

void batch_release(void* p) {
  BatchState* b = static_cast<BatchState*>(p);
  if (!b) return;
  for (BatchLane& l : b->lanes) {
    if (l.st) cudaStreamDestroy(l.st);
    if (l.done) cudaEventDestroy(l.done);
    if (l.em) cudaStreamDestroy(l.em);
    if (l.em_done) cudaEventDestroy(l.em_done);
    cudaFree(l.ws);
    cudaFree(l.Xc);
    cudaFree(l.Cc);
  }
  for (MeshBuffers& m : b->meshes) m.release();
  for (cudaEvent_t ev : b->ev_count) cudaEventDestroy(ev);
  if (b->h_tot) cudaFreeHost(b->h_tot);
  if (b->h_rmax) cudaFreeHost(b->h_rmax);
  cudaFree(b->d_rmax);
  if (b->h_ext) cudaFreeHost(b->h_ext);
  cudaFree(b->d_ext);
  if (b->h_filter) cudaFreeHost(b->h_filter);
  cudaFree(b->d_filter);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->cap_st) cudaStreamDestroy(b->cap_st);
  if (b->ev_in) cudaEventDestroy(b->ev_in);
  if (b->ev_out) cudaEventDestroy(b->ev_out);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->arena);
  for (auto& gs : b->groups)
    for (DpxGroup* g : gs) dpx_group_free(g);
  delete b;
}

static uint64_t mix(uint64_t h, uint64_t v) {
  h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
  return h;
}

static uint64_t signature(int n, const gm_batch_item* it, const std::vector<int>& ext, int mode, int se, int lanes) {
  uint64_t h = mix(0, (uint64_t)n);
  h = mix(h, (uint64_t)mode);
  h = mix(h, (uint64_t)se);
  h = mix(h, (uint64_t)lanes);
  for (int i = 0; i < n; i++) {
    h = mix(h, (uint64_t)it[i].desc.res);
    for (int a = 0; a < 3; a++) h = mix(h, (uint64_t)it[i].desc.data_res[a]);
    h = mix(h, (uint64_t)(uintptr_t)it[i].d_input);
    h = mix(h, (uint64_t)(uintptr_t)it[i].d_scale);
    h = mix(h, (uint64_t)(uintptr_t)it[i].d_closing);
    h = mix(h, (uint64_t)it[i].uniform_radius);
    h = mix(h, (uint64_t)ext[i]);
  }
  return h;
}

static cudaError_t ensure_lanes(BatchState* b, int L) {
  while ((int)b->lanes.size() < L) {
    BatchLane l;
    cudaError_t e = cudaStreamCreateWithFlags(&l.st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    e = cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
    e = cudaStreamCreateWithFlags(&l.em, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    e = cudaEventCreateWithFlags(&l.em_done, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
    b->lanes.push_back(l);
  }
  cudaError_t e = cudaSuccess;
  if (!b->fork && (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess) return e;
  if (!b->cap_st && (e = cudaStreamCreateWithFlags(&b->cap_st, cudaStreamNonBlocking)) != cudaSuccess) return e;
  if (!b->ev_in && (e = cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming)) != cudaSuccess) return e;
  if (!b->ev_out && (e = cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming)) != cudaSuccess) return e;
  return cudaSuccess;
}

// largest grids first onto the least-loaded lane
static std::vector<int> assign(int n, const std::vector<int>& ext, int L) {
  std::vector<int> order(n), lane(n, 0);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ext[a] > ext[b]; });
  std::vector<double> load(L, 0.0);
  for (int i : order) {
    int best = 0;
    for (int l = 1; l < L; l++)
      if (load[l] < load[best]) best = l;
    lane[i] = best;
    load[best] += (double)ext[i] * ext[i] * ext[i];
  }
  return lane;
}

// Closing arguments of grid i on the extent E (crop buffers Xc / Cc when the
// extent is smaller than the grid).
static CloseArgs batch_close_args(const gm_batch_item& it, int E, int rmax, int mode, int se, uint8_t* ws,
                                  uint8_t* Xc, uint8_t* Cc, int sms) {
  const bool crop = E < it.desc.res;
  CloseArgs a;
  a.res = E;
  for (int k = 0; k < 3; k++) a.data_res[k] = it.desc.data_res[k] < E ? it.desc.data_res[k] : E;
  a.X = crop ? Xc : it.d_input;
  a.R = it.d_scale;
  if (crop) {
    // the radius field is read in place, with the instance grid's strides
    a.r_sy = 2 * (int64_t)it.desc.res;
    a.r_sz = 4 * (int64_t)it.desc.res * it.desc.res;
  }
  a.uniform_r = it.uniform_radius;
  a.rmax = rmax;
  a.mode = mode;
  a.se = se;
  a.C_out = crop ? Cc : it.d_closing;
  a.D_out = nullptr;
  a.S_out = nullptr;
  a.workspace = ws;
  a.num_sms = sms;
  return a;
}

// The closing phase: fork from `st`, every lane runs its instances, join.
// With `ma`, each closing is followed on its lane by the mesh counts of the
// grid (totals to the pinned b->h_tot) and the grid's event, so that its
// emission can start while the lane goes on closing other grids.
static cudaError_t enqueue_closings(BatchState* b, int n, const gm_batch_item* it, const int* rmax,
                                    const std::vector<int>& ext, int mode, int se, int L, const std::vector<int>& lane,
                                    int sms, cudaStream_t st, KernelCounter* kc, const MeshArgs* ma = nullptr) {
  cudaError_t e = cudaEventRecord(b->fork, st);
  if (e != cudaSuccess) return e;
  for (int l = 0; l < L; l++)
    if ((e = cudaStreamWaitEvent(b->lanes[l].st, b->fork, 0)) != cudaSuccess) return e;
  for (int i = 0; i < n; i++) {
    BatchLane& ln = b->lanes[lane[i]];
    const int res = it[i].desc.res, E = ext[i];
    const bool crop = E < res;
    if (crop) {
      const int zero[3] = {0, 0, 0}, e3[3] = {E, E, E};
      if ((e = launch_box_copy(it[i].d_input, res, zero, ln.Xc, E, zero, e3, ln.st, kc)) != cudaSuccess) return e;
    }
    const CloseArgs a = batch_close_args(it[i], E, rmax[i], mode, se, ln.ws, ln.Xc, ln.Cc, sms);
    if ((e = launch_close(a, ln.st, kc)) != cudaSuccess) return e;
    if (crop && (e = launch_embed(ln.Cc, E, it[i].d_closing, res, ln.st, kc)) != cudaSuccess) return e;
    if (ma) {
      if ((e = mesh_count_launch(ma[i], b->meshes[i], ln.st, kc, b->h_tot + 4 * i)) != cudaSuccess) return e;
      // an external event node when captured: the host waits on it after the replay
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if ((e = cudaStreamIsCapturing(ln.st, &cs)) != cudaSuccess) return e;
      if ((e = cudaEventRecordWithFlags(b->ev_count[i], ln.st,
                                        cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal
                                                                            : cudaEventRecordDefault)) != cudaSuccess)
        return e;
    }
  }
  for (int l = 0; l < L; l++) {
    if ((e = cudaEventRecord(b->lanes[l].done, b->lanes[l].st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st, b->lanes[l].done, 0)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Grouped form: the closings go phase by phase (close_phases); the kernels
// of a phase run per grid on the lanes, then the phase's min-plus pass of
// all the grids as one persistent launch on `st` (dpx_group_launch: its
// blocks pull the tiles of every grid from one work counter).  Each grid
// has its own workspace in the arena.  `set` selects the pass tables: 0
// for live runs, 1 for the tables a captured graph keeps reading.
static cudaError_t enqueue_closings_grouped(BatchState* b, int set, int n, const gm_batch_item* it, const int* rmax,
                                            const std::vector<int>& ext, int mode, int se, int L,
                                            const std::vector<int>& lane, int sms, cudaStream_t st, KernelCounter* kc,
                                            const MeshArgs* ma = nullptr) {
  cudaError_t e;
  const int P = close_phases(mode);
  for (int p = 0; p < P; p++) {
    if ((e = cudaEventRecord(b->fork, st)) != cudaSuccess) return e;
    for (int l = 0; l < L; l++)
      if ((e = cudaStreamWaitEvent(b->lanes[l].st, b->fork, 0)) != cudaSuccess) return e;
    DpxGroup* g = b->groups[set][p];
    dpx_group_clear(g);
    for (int i = 0; i < n; i++) {
      BatchLane& ln = b->lanes[lane[i]];
      const int res = it[i].desc.res, E = ext[i];
      const bool crop = E < res;
      uint8_t* ws = b->arena + b->arena_off[i];
      uint8_t* Xc = crop ? ws + ((close_workspace_bytes(E) + 255) & ~(size_t)255) : nullptr;
      uint8_t* Cc = crop ? Xc + (((size_t)E * E * E + 255) & ~(size_t)255) : nullptr;
      if (p == 0 && crop) {
        const int zero[3] = {0, 0, 0}, e3[3] = {E, E, E};
        if ((e = launch_box_copy(it[i].d_input, res, zero, Xc, E, zero, e3, ln.st, kc)) != cudaSuccess) return e;
      }
      CloseArgs a = batch_close_args(it[i], E, rmax[i], mode, se, ws, Xc, Cc, sms);
      a.phase = p;
      a.group = g;
      if ((e = launch_close(a, ln.st, kc)) != cudaSuccess) return e;
      if (p == P - 1) {
        if (crop && (e = launch_embed(Cc, E, it[i].d_closing, res, ln.st, kc)) != cudaSuccess) return e;
        if (ma) {
          if ((e = mesh_count_launch(ma[i], b->meshes[i], ln.st, kc, b->h_tot + 4 * i)) != cudaSuccess) return e;
          cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
          if ((e = cudaStreamIsCapturing(ln.st, &cs)) != cudaSuccess) return e;
          if ((e = cudaEventRecordWithFlags(b->ev_count[i], ln.st,
                                            cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal
                                                                                : cudaEventRecordDefault)) !=
              cudaSuccess)
            return e;
        }
      }
    }
    for (int l = 0; l < L; l++) {
      if ((e = cudaEventRecord(b->lanes[l].done, b->lanes[l].st)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(st, b->lanes[l].done, 0)) != cudaSuccess) return e;
    }
    if (p < P - 1 && (e = dpx_group_launch(g, sms, st, kc)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Per-grid workspaces of the grouped form (grown when a batch needs more)
// and the pass tables of its phases.
static cudaError_t ensure_arena(BatchState* b, int n, const gm_batch_item* it, const std::vector<int>& ext, int mode) {
  b->arena_off.assign(n, 0);
  size_t total = 0;
  for (int i = 0; i < n; i++) {
    b->arena_off[i] = total;
    size_t sz = (close_workspace_bytes(ext[i]) + 255) & ~(size_t)255;
    if (ext[i] < it[i].desc.res) sz += 2 * ((((size_t)ext[i] * ext[i] * ext[i]) + 255) & ~(size_t)255);
    total += sz;
  }
  cudaError_t e;
  if (b->arena_bytes < total) {
    cudaFree(b->arena);
    b->arena = nullptr;
    b->arena_bytes = 0;
    if (b->inject_fail > 0) {
      b->inject_fail--;
      return cudaErrorMemoryAllocation;
    }
    if ((e = cudaMalloc(&b->arena, total)) != cudaSuccess) return e;
    b->arena_bytes = total;
  }
  const int P = close_phases(mode);
  for (auto& gs : b->groups)
    while ((int)gs.size() < P) gs.push_back(dpx_group_new());
  for (auto& gs : b->groups)
    for (int p = 0; p < P; p++)
      if ((e = dpx_group_reserve(gs[p], n)) != cudaSuccess) return e;
  return cudaSuccess;
}

// a lane buffer, or the injected out-of-memory failure
static cudaError_t lane_malloc(BatchState* b, void** p, size_t bytes) {
  if (b->inject_fail > 0) {
    b->inject_fail--;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

void batch_inject_alloc_failures(void** state, int count) {
  if (!*state) *state = new BatchState();
  static_cast<BatchState*>(*state)->inject_fail = count;
}

cudaError_t batch_run(void** state, int n, const gm_batch_item* it, int mode, int se, int bilateral, int lanes_req,
                      gm_mesh_view* meshes, int sms, cudaStream_t st, KernelCounter* kc) {
  if (!*state) *state = new BatchState();
  BatchState* b = static_cast<BatchState*>(*state);
  cudaError_t e;
  // radius bounds: uniform radii are known; radius fields are reduced on
  // the device in one round trip for the whole batch
  std::vector<int> rmax(n);
  bool all_uniform = true;
  for (int i = 0; i < n; i++) {
    rmax[i] = clamp_radius(it[i].uniform_radius);
    if (it[i].d_scale) all_uniform = false;
  }
  if (!all_uniform && b->rmax_cap < n) {
    cudaFree(b->d_rmax);
    if (b->h_rmax) cudaFreeHost(b->h_rmax);
    b->d_rmax = nullptr;
    b->h_rmax = nullptr;
    if ((e = cudaMalloc(&b->d_rmax, sizeof(int) * n)) != cudaSuccess) return e;
    if ((e = cudaMallocHost(&b->h_rmax, sizeof(int) * n)) != cudaSuccess) return e;
    b->rmax_cap = n;
  }
  if (b->ext_cap < n) {
    cudaFree(b->d_ext);
    if (b->h_ext) cudaFreeHost(b->h_ext);
    b->d_ext = nullptr;
    b->h_ext = nullptr;
    if ((e = cudaMalloc(&b->d_ext, sizeof(unsigned) * 3 * n)) != cudaSuccess) return e;
    if ((e = cudaMallocHost(&b->h_ext, sizeof(unsigned) * 3 * n)) != cudaSuccess) return e;
    b->ext_cap = n;
  }
  // one round trip: radius bounds of radius fields, occupied extents
  for (int i = 0; i < n; i++) {
    const int64_t cells = (int64_t)it[i].desc.res * it[i].desc.res * it[i].desc.res;
    if (it[i].d_scale) {
      if ((e = launch_rmax(it[i].d_scale, 8 * cells, b->d_rmax + i, sms, st, kc)) != cudaSuccess) return e;
      if ((e = cudaMemcpyAsync(b->h_rmax + i, b->d_rmax + i, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    }
    if ((e = launch_occ_extent(it[i].d_input, it[i].desc.res, b->d_ext + 3 * i, sms, st, kc)) != cudaSuccess) return e;
  }
  if ((e = cudaMemcpyAsync(b->h_ext, b->d_ext, sizeof(unsigned) * 3 * n, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  for (int i = 0; i < n; i++)
    if (it[i].d_scale) rmax[i] = b->h_rmax[i];
  // closing extents: occupied cells + dilation reach ((r+1) fine, one block
  // cell, one contour cell, one to spare), a multiple of 32 cells
  std::vector<int> ext(n);
  for (int i = 0; i < n; i++) {
    const unsigned* x = b->h_ext + 3 * i;
    const int occ = (int)std::max(x[0], std::max(x[1], x[2]));
    const int reach = occ == 0 ? 0 : occ + (rmax[i] + 2) / 2 + 3;
    int E = (std::max(reach, 32) + 31) / 32 * 32;
    if (se == GM_SE_CUBE) E = (std::max(reach + 1, 32) + 31) / 32 * 32;
    ext[i] = E >= it[i].desc.res ? it[i].desc.res : E;
  }
  // form: the lane count requested (> 0), the grouped form (kBatchGrouped),
  // or the one tuned for this signature (tuned now on its first call)
  int L = lanes_req;
  const uint64_t tune_sig = signature(n, it, ext, mode, se, 0);
  if (L == 0) {
    auto f = b->tuned.find(tune_sig);
    if (f != b->tuned.end()) L = f->second;
  }
  const bool tune = L == 0;
  bool phase_ok = true;
  for (int i = 0; i < n; i++) phase_ok = phase_ok && close_phase_ok(rmax[i], se);
  if (L == kBatchGrouped && !phase_ok) return cudaErrorNotSupported;  // a radius bound > 91
  const int cands[5] = {1, 2, 4, 8, 16};
  const int maxL = tune ? 16 : L == kBatchGrouped ? std::min(kGroupedLanes, n) : std::max(1, std::min(L, 64));
  if ((e = ensure_lanes(b, maxL)) != cudaSuccess) return e;
  // the grouped form's per-grid workspaces (a candidate of the tuner only
  // when they fit)
  bool grouped_ok = phase_ok && (tune || L == kBatchGrouped);
  if (grouped_ok && (e = ensure_arena(b, n, it, ext, mode)) != cudaSuccess) {
    if (L == kBatchGrouped) return e;
    cudaGetLastError();
    grouped_ok = false;
  }
  // per-lane workspaces and crop buffers sized for the largest closing
  int maxres = 16, maxcrop = 0;
  for (int i = 0; i < n; i++) {
    maxres = std::max(maxres, ext[i]);
    if (ext[i] < it[i].desc.res) {
      maxcrop = std::max(maxcrop, ext[i]);
    }
  }
  const size_t wsb = close_workspace_bytes(maxres);
  const size_t ccells = (size_t)maxcrop * maxcrop * maxcrop;
  for (int l = 0; l < (L == kBatchGrouped ? 0 : maxL); l++) {
    BatchLane& ln = b->lanes[l];
    if (ln.ws_bytes < wsb) {
      cudaFree(ln.ws);
      ln.ws = nullptr;
      ln.ws_bytes = 0;
      if ((e = lane_malloc(b, (void**)&ln.ws, wsb)) != cudaSuccess) return e;
      ln.ws_bytes = wsb;
    }
    if (ln.crop_cells < ccells) {
      cudaFree(ln.Xc);
      cudaFree(ln.Cc);
      ln.Xc = ln.Cc = nullptr;
      ln.crop_cells = 0;
      if ((e = lane_malloc(b, (void**)&ln.Xc, ccells)) != cudaSuccess) return e;
      if ((e = lane_malloc(b, (void**)&ln.Cc, ccells)) != cudaSuccess) return e;
      ln.crop_cells = ccells;
    }
  }
  if (tune) {
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float best_ms = 1e30f;
    int best = 1;
    std::vector<int> forms(cands, cands + 5);
    if (grouped_ok) forms.push_back(kBatchGrouped);
    for (int c : forms) {
      const int cl = c == kBatchGrouped ? std::min(kGroupedLanes, n) : c;
      const std::vector<int> lane = assign(n, ext, cl);
      // one untimed pass (first-touch, function attributes), one timed
      for (int rep = 0; rep < 2; rep++) {
        cudaEventRecord(t0, st);
        e = c == kBatchGrouped
                ? enqueue_closings_grouped(b, 0, n, it, rmax.data(), ext, mode, se, cl, lane, sms, st, nullptr)
                : enqueue_closings(b, n, it, rmax.data(), ext, mode, se, c, lane, sms, st, nullptr);
        if (e != cudaSuccess) {
          cudaEventDestroy(t0);
          cudaEventDestroy(t1);
          return e;
        }
        cudaEventRecord(t1, st);
      }
      cudaEventSynchronize(t1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, t0, t1);
      if (ms < best_ms) { best_ms = ms; best = c; }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    L = best;
    b->tuned[tune_sig] = L;
    b->last_tuned = L;
  }
  const bool grouped = L == kBatchGrouped;
  const int LL = grouped ? std::min(kGroupedLanes, n) : L;  // lanes in use
  const std::vector<int> lane = assign(n, ext, LL);
  // mesh arguments, count buffers, pinned totals and per-grid events, all
  // allocated before the closing phase (which may be captured)
  std::vector<MeshArgs> ma;
  if (meshes) {
    if ((int)b->meshes.size() < n) b->meshes.resize(n);
    b->nv.assign(n, 0);
    b->nt.assign(n, 0);
    if (b->h_tot_cap < n) {
      if (b->h_tot) cudaFreeHost(b->h_tot);
      b->h_tot = nullptr;
      if ((e = cudaMallocHost(&b->h_tot, sizeof(uint32_t) * 4 * n)) != cudaSuccess) return e;
      b->h_tot_cap = n;
    }
    while ((int)b->ev_count.size() < n) {
      cudaEvent_t ev;
      if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return e;
      b->ev_count.push_back(ev);
    }
    ma.resize(n);
    for (int i = 0; i < n; i++) {
      MeshArgs& a = ma[i];
      a.res = it[i].desc.res;
      a.C = it[i].d_closing;
      for (int k = 0; k < 3; k++) a.bbox_min[k] = it[i].desc.bbox_min[k];
      a.cell_size = it[i].desc.cell_size;
      a.isovalue = 0.95f;
      a.bilateral_iters = bilateral;
      a.defer_filter = bilateral > 0;  // filtered below, all grids per launch
      a.num_sms = sms;
      // the closing is empty beyond the extent: mesh only its cells (the
      // whole grid's border rule, identical mesh)
      a.gres = a.res;
      for (int k = 0; k < 3; k++) {
        a.tag_lo[k] = a.emit_lo[k] = 0;
        a.tag_hi[k] = a.emit_hi[k] = ext[i];
      }
      if ((e = mesh_prepare_grid(a, b->meshes[i])) != cudaSuccess) return e;
    }
  }
  // closing phase (with the mesh counts): replay the captured graph when the
  // batch is unchanged
  uint64_t sig = signature(n, it, ext, mode, se, L);
  if (meshes) {
    sig = mix(sig, (uint64_t)(uintptr_t)b->h_tot);
    for (int i = 0; i < n; i++) sig = mix(sig, (uint64_t)(uintptr_t)b->meshes[i].brick_tot);
  }
  const bool graphable = all_uniform && !(kc && kc->profiling);
  if (graphable) {
    if (!b->graph || b->graph_sig != sig) {
      if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
      }
      cudaGraph_t g = nullptr;
      KernelCounter cap;  // counts the kernels the graph holds
      // no replay of the earlier graph may still read the pass tables that
      // this capture rewrites
      if ((e = cudaEventSynchronize(b->ev_out)) != cudaSuccess) return e;
      if ((e = cudaStreamBeginCapture(b->cap_st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
      const cudaError_t ec =
          grouped ? enqueue_closings_grouped(b, 1, n, it, rmax.data(), ext, mode, se, LL, lane, sms, b->cap_st, &cap,
                                             meshes ? ma.data() : nullptr)
                  : enqueue_closings(b, n, it, rmax.data(), ext, mode, se, L, lane, sms, b->cap_st, &cap,
                                     meshes ? ma.data() : nullptr);
      e = cudaStreamEndCapture(b->cap_st, &g);
      if (ec != cudaSuccess) return ec;
      if (e != cudaSuccess) return e;
      e = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return e;
      b->graph_sig = sig;
      b->graph_kernels = cap.launches;
    }
    if ((e = cudaEventRecord(b->ev_in, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(b->cap_st, b->ev_in, 0)) != cudaSuccess) return e;
    if ((e = cudaGraphLaunch(b->graph, b->cap_st)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(b->ev_out, b->cap_st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st, b->ev_out, 0)) != cudaSuccess) return e;
    if (kc) kc->launches += b->graph_kernels;
  } else {
    e = grouped ? enqueue_closings_grouped(b, 0, n, it, rmax.data(), ext, mode, se, LL, lane, sms, st, kc,
                                           meshes ? ma.data() : nullptr)
                : enqueue_closings(b, n, it, rmax.data(), ext, mode, se, L, lane, sms, st, kc,
                                   meshes ? ma.data() : nullptr);
    if (e != cudaSuccess) return e;
  }
  if (!meshes) return cudaGetLastError();
  // meshing: each grid's emission, on its lane's emission stream, once its
  // counts are on the host (the closings of later grids go on meanwhile)
  for (int i = 0; i < n; i++) {
    if ((e = cudaEventSynchronize(b->ev_count[i])) != cudaSuccess) return e;
    if ((e = mesh_count_finish(b->meshes[i], b->h_tot + 4 * i, &b->nv[i], &b->nt[i])) != cudaSuccess) return e;
    if (b->nv[i] > 0xfffffff0LL || b->nt[i] > 0x7ffffff0LL) return cudaErrorInvalidValue;
    cudaStream_t em = b->lanes[lane[i]].em;
    if ((e = cudaStreamWaitEvent(em, b->ev_count[i], 0)) != cudaSuccess) return e;
    if ((e = mesh_emit(ma[i], b->meshes[i], b->nv[i], b->nt[i], em, kc)) != cudaSuccess) return e;
    meshes[i].vertices = b->meshes[i].V;
    meshes[i].normals = b->meshes[i].N;
    meshes[i].triangles = b->meshes[i].T;
    meshes[i].num_vertices = b->nv[i];
    meshes[i].num_triangles = b->nt[i];
  }
  for (int l = 0; l < LL; l++) {
    cudaEventRecord(b->lanes[l].em_done, b->lanes[l].em);
    cudaStreamWaitEvent(st, b->lanes[l].em_done, 0);
  }
  if (bilateral > 0) {
    // normal filtering of all the meshes, one launch per iteration (the
    // host table is free again: the previous call's copy of it preceded this
    // call's closings on st, which the waits for the grids' counts above
    // followed)
    if (b->filter_cap < n) {
      if (b->h_filter) cudaFreeHost(b->h_filter);
      cudaFree(b->d_filter);
      b->h_filter = nullptr;
      b->d_filter = nullptr;
      b->filter_cap = 0;
      if ((e = cudaMallocHost(&b->h_filter, mesh_filter_table_bytes(n))) != cudaSuccess) return e;
      if ((e = cudaMalloc(&b->d_filter, mesh_filter_table_bytes(n))) != cudaSuccess) return e;
      b->filter_cap = n;
    }
    std::vector<MeshBuffers*> mp(n);
    std::vector<int> zi(n, 0);
    for (int i = 0; i < n; i++) mp[i] = &b->meshes[i];
    if ((e = mesh_filter_group(mp.data(), b->nv.data(), zi.data(), n, bilateral, b->d_filter, b->h_filter, sms, st,
                               kc)) != cudaSuccess)
      return e;
  }
  return cudaGetLastError();
}

int batch_lanes_tuned(void* state) {
  BatchState* b = static_cast<BatchState*>(state);
  return b ? b->last_tuned : 0;
}

}  // namespace gm
